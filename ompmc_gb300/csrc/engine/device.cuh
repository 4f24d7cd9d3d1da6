// Device-side building blocks of the transport engine: precision traits,
// RANMAR streams, per-lane particle stacks, resident tables and the voxel
// geometry.  Physics lives in physics.cuh.
#pragma once

#include <cstdint>

#include "omc_gpu.h"

namespace omcgpu {

constexpr int MXGE = OMC_MXGE;
constexpr int MXEKE = OMC_MXEKE;
constexpr int MXRAYFF = OMC_MXRAYFF;
constexpr int MXE_SPIN = OMC_MXE_SPIN;
constexpr int MXE_SPIN1 = OMC_MXE_SPIN1;
constexpr int MXQ_SPIN = OMC_MXQ_SPIN;
constexpr int MXU_SPIN = OMC_MXU_SPIN;
constexpr int MXL_MS = OMC_MXL_MS;
constexpr int MXQ_MS = OMC_MXQ_MS;
constexpr int MXU_MS = OMC_MXU_MS;
constexpr int RNG_WORDS = 97;

// Device error bits (omc_run_stats.error_flags).
enum : unsigned {
  ERR_STACK = 1u,      // per-lane stack overflow: history dropped
  ERR_LOOP = 2u,       // a rejection loop hit its iteration cap
  ERR_EVENTS = 4u,     // a history exceeded the event cap: history dropped
  ERR_TABLE = 8u,      // an interpolation index left its table (clamped)
  ERR_QUEUE = 16u,     // wavefront queue full: particle dropped
  ERR_BARRIER = 32u,   // a grid barrier gave up waiting
  ERR_HISTORY = 64u    // history-by-history scoring: block pool empty or a
                       // history over its region limit (its sums are split)
};

// Iteration caps of device loops.  The reference's loops end with
// probability one; the caps only turn a pathological input into an error
// flag instead of a hung GPU.
constexpr int kRejectCap = 1 << 20;
constexpr long long kEventCap = 1ll << 22;
// A photon flight with no crossing cap (split photons, the per-lane
// schedule, the end-of-run drain).
constexpr int kNoFlightCap = 1 << 30;

// ---------------------------------------------------------------------------
// Particles.  dnear is not carried: the reference writes it but never reads
// it (ompmc.c:4934-4935, 5109, 5254).
template <typename R>
struct Particle {
  R e, x, y, z, u, v, w, wt;
  int iq, ir;
};

// Four table values read together (one 16- or 32-byte load).
template <typename R>
struct alignas(4 * sizeof(R)) V4 {
  R x, y, z, w;
};

// ---------------------------------------------------------------------------
// Tables resident on the device, converted to R.  Scalar arrays keep the
// reference's index layout (the arrays of omc_tables); the interpolation
// coefficients read on every step are also packed per (medium, energy bin)
// into V4 records so that a lookup is one load:
//   ph_mfp [m][l] = {gmfp1, gmfp0, cohe1, cohe0}
//   ph_br  [m][l] = {gbr11, gbr10, gbr21, gbr20}
//   el_sd  [q][m][l] = {sig1, sig0, dedx1, dedx0}   (q = 0 e-, 1 e+)
//   el_te  [q][m][l] = {tmxs1, tmxs0, eta1, eta0}
//   el_rg  [q][m][l] = {blcce1, blcce0, range_ep, e_array}
//   el_q   [q][m][l] = {q1c1, q1c0, q2c1, q2c0}
//   el_ib  [m][l] = {ebr11, ebr10, pbr11, pbr10},  el_ib2 [m][l] = {pbr21, pbr20, 0, 0}
template <typename R>
struct Tables {
  const V4<R> *ph_mfp, *ph_br, *el_sd, *el_te, *el_rg, *el_q, *el_ib, *el_ib2;
  int nmed;
  // per medium
  const R *ge0, *ge1, *eke0, *eke1, *xcc, *blcc, *te, *thmoll, *ap;
  const R *esig_e, *psig_e, *delcm, *zbrang, *bpar0, *bpar1;
  const int *monotone;  // [2*nmed]
  // photon [nmed*MXGE]
  const R *gmfp0, *gmfp1, *gbr10, *gbr11, *gbr20, *gbr21, *cohe0, *cohe1, *pmax0, *pmax1;
  // rayleigh [MXRAYFF] of medium 0 (see rayleigh())
  const R *xgrid, *fcum, *b_array, *c_array;
  const int *i_array;
  // pair/brems [nmed*8]
  const R *dl1, *dl2, *dl3, *dl4, *dl5, *dl6;
  // electron [nmed*MXEKE]
  const R *esig0, *esig1, *psig0, *psig1, *ededx0, *ededx1, *pdedx0, *pdedx1;
  const R *ebr10, *ebr11, *pbr10, *pbr11, *pbr20, *pbr21, *tmxs0, *tmxs1, *blcce0, *blcce1;
  const R *etae0, *etae1, *etap0, *etap1, *q1ce0, *q1ce1, *q1cp0, *q1cp1, *q2ce0, *q2ce1, *q2cp0, *q2cp1;
  const R *e_array, *range_ep;  // range_ep [2*nmed*MXEKE]
  const int *meke;              // [nmed]
  // spin
  R b2spin_min, dbeta2i, espml, dleneri, dqq1i;
  const R *spin_rej;
  // msnew
  const R *ums, *fms, *wms;
  const int *ims;
  R dllambi, dqmsi;
};

// Voxel geometry and per-region data.
// Unsigned division by a divisor fixed for a whole run, as a multiply-high
// and shifts (Granlund and Montgomery, "Division by invariant integers
// using multiplication", PLDI 1994, round-up method with a 33-bit
// multiplier): exact for every 32-bit dividend.  l = 0 marks d = 1.
struct InvariantDivisor {
  unsigned m;
  int l;
};

inline InvariantDivisor make_divisor(unsigned d) {
  if (d <= 1) return InvariantDivisor{0u, 0};
  int l = 0;
  while ((1ull << l) < d) l++;  // ceil(log2 d)
  unsigned long long m = (((1ull << 32) * ((1ull << l) - d)) / d) + 1;
  return InvariantDivisor{static_cast<unsigned>(m), l};
}

__device__ __forceinline__ unsigned divide(unsigned n, InvariantDivisor v) {
  if (v.l == 0) return n;
  unsigned t = __umulhi(v.m, n);
  return (t + ((n - t) >> 1)) >> (v.l - 1);
}

// Per-voxel transport data in one record.
template <typename R>
struct alignas(2 * sizeof(R)) VoxelRec {
  R rhof;   // density / density of the medium in the pegs4 data
  int med;  // medium index, -1 = vacuum (region 0, outside the phantom)
};

template <typename R>
struct Geometry {
  int nx, ny, nz, nxy;
  InvariantDivisor div_nx, div_nxy;  // region decode (omc_dosxyz.c:205-207)
  const R *xb, *yb, *zb;
  // [nreg] voxel records {rhof, medium (-1 vacuum / outside)}: one
  // 8-byte (FP32) or 16-byte (FP64) load per voxel visited
  const VoxelRec<R> *vox;
  const R *ecut_m, *pcut_m;  // per medium (+1 slot for vacuum at index 0)
};

// Source (initSource, omc_dosxyz.c:368-632) in R.  With beamlets set
// (omc_matrad.c:543-750) histories start on a beamlet's bixel instead of
// the collimated point source.
template <typename R>
struct Source {
  int spectrum, charge;
  R energy, deltak;
  const R *cdfinv1, *cdfinv2;  // [INVDIM]
  R ssd, xinl, yinl, xsize, ysize;
  int ixinl, iyinl;
  int beamlets;        // 1: beamlet source
  const R *bixel;      // [nbeamlets][9] corner xyz, side1 xyz, side2 xyz
  const R *beam_src;   // [nbeams][3] source point of each beam
  const int *ibeam;    // [nbeamlets]
};

// One resident dose job of a multi-job launch: its own phantom, source,
// tallies and source-energy sum.  Field jobs: history k of the job
// (counted over all launches) scores in batch k / nperbatch.  Beamlet
// (dij) jobs: history k belongs to the beamlet b with bl_first[b] <= k <
// bl_first[b+1], starts from that beamlet's source, and scores in tally b.
template <typename R>
struct JobSlot {
  Geometry<R> G;
  Source<R> S;
  double *tally;        // [nbatch][nreg], beamlet jobs [nbl][nreg]
  double *ensrc;        // [1]
  long long nreg;
  long long h0;         // job history index of this launch's first history
  long long nperbatch;
  const long long *bl_first;  // beamlet jobs: [nbl + 1] first job history of each beamlet
  int nbl;                    // beamlets (0: field job)
};

// Queue tag of a particle in a multi-job launch: job slot and batch (or
// beamlet).
constexpr int kBatchTag = 4096;

// History-by-history scoring (wavefront schedule, optional).  Every
// history in flight owns a chain of blocks from a pool; its particles carry
// the head block in their queue tag, each deposit appends (region, energy)
// to the chain, and the head block counts the history's particles in flight.
// When a take brings that count to zero, the lane's warp merges the chain
// by region (all 32 lanes on one history, in a shared-memory table) and
// adds the history's energy x in each region to sum[r] and x^2 to sum2[r]
// -- the history-by-history estimators of Walters, Kawrakow and Rogers
// (Med. Phys. 29 (2002) 2745) -- then returns the blocks.  Blocks of 384
// bytes: a 16-byte header and (region, energy) entries.
constexpr int kHbhBlockBytes = 384;
constexpr int kHbhRegions = 128;  // distinct regions of one history the warp's merge table holds
template <typename R>
struct HbhBlock {
  static constexpr int kEntries = (kHbhBlockBytes - 16) / static_cast<int>(4 + sizeof(R));
  int count;  // entries appended; those past kEntries went to the next block
  int next;   // continuation block, -1 none
  int live;   // head block: particles of the history queued or being processed
  int slot;   // head block: tally slot (batch) of the history
  int ir[kEntries];
  R x[kEntries];
};

// Free blocks: a ring of block ids with a push and a pop counter.  A pop
// in a wavefront iteration only takes entries pushed before the iteration
// began (their writes are complete), so it never reads an entry that a
// concurrent push is writing; the ring never holds more than nblocks ids,
// so a push never overwrites an entry that is still to be popped.
template <typename R>
struct HbhPool {
  HbhBlock<R> *blocks;
  int nblocks;
  int *ring;                  // [ring_mask + 1], a power of two >= nblocks
  unsigned ring_mask;
  unsigned long long *ctr;    // {ids pushed, ids popped}
  double *sum, *sum2;         // [nreg] sums over histories of x and x^2
  unsigned long long *histories;  // histories merged
  unsigned long long *split;      // histories merged in parts (over the local region table)
};

template <typename R>
struct Params {
  Tables<R> T;
  Geometry<R> G;
  Source<R> S;
  int nsplit;
  int nlanes;
  int depth;                 // per-lane stack slots
  long long nhist;           // histories of this launch
  unsigned long long *next;  // history counter
  // per-lane state in HBM
  int *rng_u;                // [97][nlanes]
  int *rng_ijc;              // [3][nlanes]
  R *stk;                    // [8][depth][nlanes]
  int *stk_key;              // [depth][nlanes]  ir*4 + iq+1
  // beamlet jobs: history h of the launch belongs to tally slot s with
  // slot_first[s] <= h < slot_first[s+1]; slot s scores into
  // endep[s*nreg ...] and transports beamlet slot_beamlet[s]
  int nslots;                        // 0: one tally, no beamlets
  const long long *slot_first;       // [nslots+1]
  const int *slot_beamlet;           // [nslots]
  long long tally_stride;            // nreg
  const JobSlot<R> *__restrict__ jobs;  // multi-job launches: [nslots]
  // outputs
  double *endep;             // [nreg] batch tally ([nslots][nreg] with slots)
  double *ensrc;             // [1]
  unsigned long long *events;
  unsigned long long *n_geom;
  unsigned long long *n_dep;
  int *max_np;
  unsigned *err;
  HbhPool<R> hbh;            // history-by-history scoring (blocks null: off)
};

// ---------------------------------------------------------------------------
// RANMAR (omc_random.c:58-187) with the 97-word state in shared memory.
// Every word is a 24-bit integer, kept as a 16-bit low plane and an 8-bit
// high plane (3 bytes per word instead of 4, so more lanes fit on an SM);
// word k of a thread sits at index k*stride of each plane.  Numbers are
// produced one at a time; the reference refills blocks of 128 but returns
// them in the same order.
struct Ranmar {
  unsigned short *lo;
  unsigned char *hi;
  int stride;
  int i, j, c;

  __device__ __forceinline__ int word(int k) const {
    return static_cast<int>(lo[k * stride]) | (static_cast<int>(hi[k * stride]) << 16);
  }
  __device__ __forceinline__ void set_word(int k, int v) {
    lo[k * stride] = static_cast<unsigned short>(v & 0xffff);
    hi[k * stride] = static_cast<unsigned char>(v >> 16);
  }
  __device__ __forceinline__ int next_int() {
    int iopt = word(i - 1) - word(j - 1);
    if (iopt < 0) iopt += 16777216;
    set_word(i - 1, iopt);
    i -= 1;
    j -= 1;
    if (i == 0) i = 97;
    else if (j == 0) j = 97;
    c -= 7654321;
    if (c < 0) c += 16777213;
    iopt -= c;
    if (iopt < 0) iopt += 16777216;
    return iopt;
  }
};

// Same generator on a plain int array in global memory (state words at
// u[k*stride]); used where a stream is drawn outside the transport kernels.
struct RanmarGlobal {
  int *u;
  int stride;
  int i, j, c;
  __device__ __forceinline__ int next_int() {
    int iopt = u[(i - 1) * stride] - u[(j - 1) * stride];
    if (iopt < 0) iopt += 16777216;
    u[(i - 1) * stride] = iopt;
    i -= 1;
    j -= 1;
    if (i == 0) i = 97;
    else if (j == 0) j = 97;
    c -= 7654321;
    if (c < 0) c += 16777213;
    iopt -= c;
    if (iopt < 0) iopt += 16777216;
    return iopt;
  }
};

// Seed one stream exactly as initRandom (omc_random.c:75-123).
__host__ __device__ inline void ranmar_seed(int ixx, int jxx, int *u, int stride) {
  if (ixx <= 0 || ixx > 31328) ixx = 1802;
  if (jxx <= 0 || jxx > 31328) jxx = 9373;
  int i = (ixx / 177 % 177) + 2;
  int j = (ixx % 177) + 2;
  int k = (jxx / 169 % 178) + 1;
  int l = (jxx % 169);
  for (int ii = 0; ii < 97; ii++) {
    int s = 0, t = 8388608;
    for (int jj = 0; jj < 24; jj++) {
      int m = ((i * j % 179) * k) % 179;
      i = j;
      j = k;
      k = m;
      l = (53 * l + 1) % 169;
      if (l * m % 64 >= 32) s += t;
      t /= 2;
    }
    u[ii * stride] = s;
  }
}

// Seed pair of stream k.  initRandom accepts jxx in 1..31328 but reads it
// through (jxx/169 % 178, jxx % 169), which has only 30082 distinct values:
// jxx = 30082 + r gives the same stream as jxx = r.  Stream k is therefore
// (ixx, jxx + k), the reference's OpenMP thread k (omc_random.c:72), as long
// as jxx + k <= 30081; past that it continues with the next stream not yet
// used, into ixx + 1, so that no two of 31328 * 30082 consecutive streams
// are the same.  Stream 0 is (ixx, jxx) itself.
constexpr int kJxxStreams = 30082;  // distinct streams per ixx (jxx mod 30082)
__host__ __device__ inline void stream_seeds(int ixx, int jxx, long long k, int *ik, int *jk) {
  if (ixx <= 0 || ixx > 31328) ixx = 1802;
  if (jxx <= 0 || jxx > 31328) jxx = 9373;
  if (k == 0) {
    *ik = ixx;
    *jk = jxx;
    return;
  }
  const long long lin = (long long)(jxx % kJxxStreams) + k;
  const int c = (int)(lin % kJxxStreams);
  *jk = c == 0 ? kJxxStreams : c;
  *ik = (int)(((long long)(ixx - 1) + lin / kJxxStreams) % 31328) + 1;
}

}  // namespace omcgpu
