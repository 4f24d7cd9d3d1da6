/*
 * Test oracle: a CPU restatement of the reference's transport path.
 *
 * TEST INFRASTRUCTURE ONLY.  Only tests/, __graft_entry__.smoke() and the
 * CPU-baseline leg of bench.py may load this library, as the checker (or the
 * timed CPU baseline); the product never links it.
 *
 * It restates, in FP64 and with the reference's operation order and random
 * number consumption, the omc_dosxyz history loop of edoerner/ompMC:
 * RANMAR (src/omc_random.c:58-187), initHistory (ucodes/omc_dosxyz/
 * omc_dosxyz.c:964-1068), howfar/hownear/ausgab (:187-334, :683-694),
 * shower/photon/electron and every interaction (src/ompmc.c:83-211,
 * 1102-1145, 1429-1846, 1849-2121, 3097-3199, 3606-4645, 4648-5447) and the
 * batch scoring (omc_dosxyz.c:696-717).  It reads tables built by the
 * product's host library (omc_tables_build), which are themselves pinned
 * bit-for-bit against the reference's own tables.
 *
 * With nthreads = 1 it reproduces the reference's serial build exactly (same
 * seeds, same history order); with nthreads > 1 thread t uses the seed pair
 * (ixx, jxx + t) and a dynamic history schedule, like the OpenMP build.
 */
#ifndef OMC_ORACLE_H
#define OMC_ORACLE_H

#include "omc_gpu.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct omc_oracle_result {
    double ensrc;            /* sum of source kinetic energies */
    double seconds;          /* wall time of the batch loop */
    long long histories;
    int nthreads;
    int status;              /* 0 ok, 1 stack overflow */
} omc_oracle_result;

/* Runs nbatch batches of nperbatch histories of the omc_dosxyz source.
 * accum_endep / accum_endep2 (nreg entries each) receive the batch sums
 * exactly as score.accum_endep / accum_endep2 before accumulateResults.
 * nthreads <= 0 uses every available core. */
int omc_oracle_run(const omc_tables *t, const omc_phantom *ph,
                   const omc_regions *rg, const omc_source *src, int nsplit,
                   long long nperbatch, int nbatch, int ixx, int jxx,
                   int nthreads, double *accum_endep, double *accum_endep2,
                   omc_oracle_result *res);

/* Energy deposited inside the phantom by each batch of the last
 * omc_oracle_run (at most cap values); returns how many were written. */
int omc_oracle_batch_totals(double *out, int cap);

/* The omc_matrad beamlet loop (ucodes/omc_matrad/omc_matrad.c:1374-1512):
 * beamlet by beamlet, nbatch batches of (nhist[ib] or nperbatch*nbatch)/
 * nbatch histories from the beamlet source (initHistory(ibeamlet),
 * :1084-1254), then the beamlet's dose (accumulateResults, :839-919),
 * threshold and CSC column.  out's arrays are malloc'd; release them with
 * omc_oracle_dij_free.  Returns 0 on success. */
int omc_oracle_run_dij(const omc_tables *t, const omc_phantom *ph,
                       const omc_regions *rg, const omc_source *src,
                       const omc_beamlets *bl, int nsplit,
                       const long long *nhist, long long nperbatch,
                       int nbatch, int ixx, int jxx, int nthreads,
                       double rel_threshold, omc_dij *out,
                       omc_oracle_result *res);
void omc_oracle_dij_free(omc_dij *d);

/* n numbers of the RANMAR stream seeded (ixx, jxx) as 24-bit integers. */
void omc_oracle_ranmar(int ixx, int jxx, long long n, int *out);

#ifdef __cplusplus
}
#endif
#endif
