/*
 * omc_gpu.h -- C ABI of the GB300 photon/electron voxel transport engine.
 *
 * The reference (edoerner/ompMC) is a C library whose "API" is the EGS
 * user-code contract: a front end (ucodes/omc_dosxyz/omc_dosxyz.c,
 * ucodes/omc_matrad/omc_matrad.c) parses a key/value input file, builds the
 * interaction tables with initMediaData() (src/ompmc.c:5450), and then runs
 *
 *     for batch: #pragma omp parallel for  { initHistory(); shower(); }
 *
 * (omc_dosxyz.c:1237-1263, omc_matrad.c:1389-1414) with per-step host
 * callbacks howfar/hownear/ausgab (src/ompmc.h:37-39).  Per-step host
 * callbacks cannot cross to a GPU, so the drop-in boundary here is the
 * "run N histories" call: omc_engine_run() replaces that batch/history loop,
 * and the geometry, source and scoring semantics of howfar/hownear/ausgab/
 * initHistory live on the device.  Everything else keeps the reference's
 * input formats and meaning: the .inp key/value file, .egsphant phantoms,
 * spectrum files, pegs4 media, XCOM cross sections, pgs4form form factors,
 * msnew.data and spinms.data, and the .3ddose output.
 *
 * Conventions
 *  - Plain C types only; every array is caller-visible host memory unless a
 *    function says "device".
 *  - Region index irl = 1 + ix + iy*nx + iz*nx*ny, irl = 0 is outside the
 *    phantom (omc_dosxyz.c:205-207, 735).  Per-region arrays have
 *    nx*ny*nz + 1 entries.
 *  - Every function returns omc_status; the reference's printf+exit paths
 *    become error codes with a message in omc_last_error().
 *  - Engines are not thread safe; use one engine per host thread.
 */
#ifndef OMC_GPU_H
#define OMC_GPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Table dimensions, identical to the reference (src/ompmc.h). */
#define OMC_MXMED 9          /* media per problem          ompmc.h:358 */
#define OMC_MXELEMENT 50     /* elements read from data     ompmc.h:359 */
#define OMC_MXGE 2000        /* photon log-energy bins      ompmc.h:102 */
#define OMC_MXEKE 500        /* electron log-energy bins    ompmc.h:360 */
#define OMC_MXRAYFF 100      /* Rayleigh form-factor grid   ompmc.h:130 */
#define OMC_RAYCDFSIZE 100   /* Rayleigh CDF bins           ompmc.h:131 */
#define OMC_MXE_SPIN 15      /*                             ompmc.h:257 */
#define OMC_MXE_SPIN1 31     /* 2*MXE_SPIN+1                ompmc.h:258 */
#define OMC_MXQ_SPIN 15      /*                             ompmc.h:259 */
#define OMC_MXU_SPIN 31      /*                             ompmc.h:260 */
#define OMC_MXL_MS 63        /* msnew lambda grid           ompmc.h:292 */
#define OMC_MXQ_MS 7         /* msnew q grid                ompmc.h:293 */
#define OMC_MXU_MS 31        /* msnew u grid                ompmc.h:294 */
#define OMC_INVDIM 1000      /* spectrum inverse-CDF bins   omc_dosxyz.c:340 */
#define OMC_MXEBIN 200       /* spectrum bins               omc_dosxyz.c:339 */
#define OMC_NAME_LEN 64

typedef enum omc_status {
    OMC_OK = 0,
    OMC_ERR_ARG = 1,      /* invalid argument                              */
    OMC_ERR_IO = 2,       /* file missing or unreadable                    */
    OMC_ERR_INPUT = 3,    /* required .inp key missing or malformed        */
    OMC_ERR_MEDIA = 4,    /* medium not found in the pegs4 file            */
    OMC_ERR_FORMAT = 5,   /* data file does not follow its format          */
    OMC_ERR_NOMEM = 6,    /* host or device allocation failed              */
    OMC_ERR_CUDA = 7,     /* CUDA runtime error                            */
    OMC_ERR_STACK = 8,    /* particle stack overflow on the device         */
    OMC_ERR_LIMIT = 9,    /* a bounded device loop hit its iteration limit */
    OMC_ERR_STATE = 10    /* call out of order (e.g. run before load)      */
} omc_status;

const char *omc_status_string(omc_status s);
/* Message of the most recent failing call on this host thread. */
const char *omc_last_error(void);

/* ------------------------------------------------------------------------
 * Input file.  Replaces parseInputFile/getInputValue
 * (src/omc_utilities.c:63-123): "key = value" lines, any line containing '#'
 * or only white space is skipped, keys match by SUBSTRING, first match wins.
 * ---------------------------------------------------------------------- */
typedef struct omc_input omc_input;

/* Parses "<path>.inp" (the ".inp" extension is appended, as the reference). */
omc_status omc_input_parse(const char *path_without_ext, omc_input **out);
/* Parses the same format from a string. */
omc_status omc_input_from_string(const char *text, omc_input **out);
/* 1 and the value copied to dest if found, 0 otherwise. */
int omc_input_get(const omc_input *in, const char *key, char *dest, size_t cap);
void omc_input_free(omc_input *in);

/* ------------------------------------------------------------------------
 * Phantom.  Replaces initPhantom (omc_dosxyz.c:62-175) and the MATLAB-array
 * variant of omc_matrad (omc_matrad.c:269-342).
 * ---------------------------------------------------------------------- */
typedef struct omc_phantom {
    int nmed;
    char med_names[OMC_MXMED][OMC_NAME_LEN];
    int nx, ny, nz;
    double *xbounds; /* nx+1 */
    double *ybounds; /* ny+1 */
    double *zbounds; /* nz+1 */
    int *med_index;  /* nx*ny*nz, egsphant medium number (1-based, 0 = vacuum) */
    double *density; /* nx*ny*nz, g/cm^3 */
} omc_phantom;

omc_status omc_phantom_read(const char *egsphant_path, omc_phantom **out);
omc_status omc_phantom_create(int nmed, const char *const *med_names, int nx,
                              int ny, int nz, const double *xbounds,
                              const double *ybounds, const double *zbounds,
                              const int *med_index, const double *density,
                              omc_phantom **out);
omc_status omc_phantom_write(const omc_phantom *ph, const char *egsphant_path);
void omc_phantom_free(omc_phantom *ph);

/* ------------------------------------------------------------------------
 * Media and interaction tables.  Replaces initMediaData (ompmc.c:5450):
 * readPegsFile (:5489), initPhotonData (:471), initRayleighData (:820),
 * initPairData (:1189), initMscatData (:3282) with initSpinData (:2376).
 * Field names and index layouts are the reference's globals photon_data,
 * rayleigh_data, pair_data, electron_data, spin_data, mscat_data, pegs_data
 * (ompmc.h:105-404), so values compare one to one.
 * Reads the "pegs file", "pgs4form file" and "data folder" keys.
 * ---------------------------------------------------------------------- */
typedef struct omc_tables {
    int nmed;
    char names[OMC_MXMED][OMC_NAME_LEN];
    /* pegs_data */
    int ne[OMC_MXMED], meke[OMC_MXMED];
    double rho[OMC_MXMED], rlc[OMC_MXMED], ae[OMC_MXMED], ap[OMC_MXMED];
    double ue[OMC_MXMED], up[OMC_MXMED], te[OMC_MXMED], thmoll[OMC_MXMED];
    double pegs_delcm[OMC_MXMED];
    /* photon_data: ge0/ge1 [nmed]; the rest [nmed*MXGE] */
    double *ge0, *ge1;
    double *gmfp0, *gmfp1, *gbr10, *gbr11, *gbr20, *gbr21, *cohe0, *cohe1;
    /* rayleigh_data: [nmed*MXRAYFF] except pmax [nmed*MXGE] */
    double *xgrid, *fcum, *b_array, *c_array, *pmax0, *pmax1;
    int *i_array;
    /* pair_data: dl* [nmed*8], the rest [nmed] */
    double *dl1, *dl2, *dl3, *dl4, *dl5, *dl6;
    double *bpar0, *bpar1, *delcm, *zbrang;
    /* electron_data: [nmed*MXEKE] unless noted */
    double *esig0, *esig1, *psig0, *psig1;
    double *ededx0, *ededx1, *pdedx0, *pdedx1;
    double *ebr10, *ebr11, *pbr10, *pbr11, *pbr20, *pbr21;
    double *tmxs0, *tmxs1, *blcce0, *blcce1;
    double *etae_ms0, *etae_ms1, *etap_ms0, *etap_ms1;
    double *q1ce_ms0, *q1ce_ms1, *q1cp_ms0, *q1cp_ms1;
    double *q2ce_ms0, *q2ce_ms1, *q2cp_ms0, *q2cp_ms1;
    double *e_array;
    double *range_ep;       /* [2*nmed*MXEKE], [qel][imed][i] */
    double *eke0, *eke1;    /* [nmed] */
    int *sig_ismonotone;    /* [2*nmed], [qel][imed] */
    double *esig_e, *psig_e, *xcc, *blcc, *expeke1; /* [nmed] */
    /* spin_data */
    double b2spin_min, dbeta2i, espml, dleneri, dqq1i;
    double *spin_rej; /* [nmed][2][MXE_SPIN1+1][MXQ_SPIN+1][MXU_SPIN+1] */
    /* mscat_data: [(MXL_MS+1)*(MXQ_MS+1)*(MXU_MS+1)] */
    double *ums, *fms, *wms;
    int *ims;
    double dllambi, dqmsi;
} omc_tables;

/* Builds tables for the media named in med_names (nmed entries, the
 * phantom's media list, in that order). */
omc_status omc_tables_build(const omc_input *in, int nmed,
                            const char (*med_names)[OMC_NAME_LEN],
                            omc_tables **out);
void omc_tables_free(omc_tables *t);
/* Writes every table in the "OMCT" record format used by the test oracle
 * (4-byte magic, then {u32 name length, name, u8 'd'|'i', u64 n, data}). */
omc_status omc_tables_dump(const omc_tables *t, const char *path);

/* ------------------------------------------------------------------------
 * Regions.  Replaces initRegions (omc_dosxyz.c:890-962): per region medium
 * (egsphant index - 1, -1 = vacuum), density ratio rhof, pcut, ecut.
 * Reads "global ecut" and "global pcut".  Where the reference leaves ecut
 * unset (global ecut below the pegs AE, omc_dosxyz.c:951-957) the pegs AE is
 * used, which is what its warning message announces.
 * ---------------------------------------------------------------------- */
typedef struct omc_regions {
    int nreg; /* nx*ny*nz + 1 */
    int *med;
    double *rhof, *pcut, *ecut;
} omc_regions;

omc_status omc_regions_build(const omc_input *in, const omc_phantom *ph,
                             const omc_tables *t, omc_regions **out);
void omc_regions_free(omc_regions *r);

/* ------------------------------------------------------------------------
 * Source.  Replaces initSource (omc_dosxyz.c:368-632): a point source at
 * distance "ssd" above a collimated rectangle on the phantom's z = zmin
 * face, monoenergetic ("mono energy") or from a spectrum file ("spectrum
 * file", which takes precedence), charge -1/0/+1.  Beamlet sources of
 * omc_matrad (omc_matrad.c:502-760, 1084-1254) use omc_beamlets below.
 * ---------------------------------------------------------------------- */
typedef struct omc_source {
    int spectrum; /* 0 mono, 1 spectrum */
    int charge;
    double energy;
    double deltak; /* INVDIM */
    double cdfinv1[OMC_INVDIM], cdfinv2[OMC_INVDIM];
    double ssd;
    double xinl, xinu, yinl, yinu, xsize, ysize;
    int ixinl, ixinu, iyinl, iyinu;
} omc_source;

omc_status omc_source_build(const omc_input *in, const omc_phantom *ph,
                            omc_source **out);
void omc_source_free(omc_source *s);

/* ------------------------------------------------------------------------
 * Scoring output.  Replaces accumulateResults/outputResults
 * (omc_dosxyz.c:719-886): batch mean and batch relative uncertainty, energy
 * to Gy by 1.602e-10/(rho*V*N), zero dose where density < 0.044.
 * dose/unc have nx*ny*nz+1 entries in region order (index 0 unused).
 * ---------------------------------------------------------------------- */
omc_status omc_accumulate_results(const omc_phantom *ph,
                                  const double *accum_endep,
                                  const double *accum_endep2, int iout,
                                  long long nhist, int nbatch, double *dose,
                                  double *unc);
omc_status omc_write_3ddose(const char *path, const omc_phantom *ph,
                            const double *dose, const double *unc);

/* ------------------------------------------------------------------------
 * Transport engine (GB300).  One engine owns one CUDA device context
 * slot, its resident tables, geometry and RANMAR streams.
 * ---------------------------------------------------------------------- */
typedef struct omc_engine omc_engine;

typedef enum omc_precision {
    OMC_FP64 = 0, /* FP64 transport and tallies (the reference's arithmetic) */
    OMC_FP32 = 1  /* FP32 transport arithmetic, FP64 tallies and balances   */
} omc_precision;

typedef struct omc_run_config {
    long long nperbatch; /* histories per batch                           */
    int nbatch;          /* statistical batches (omc_dosxyz.c:1214-1225)  */
    int ixx, jxx;        /* "rng seeds"; lane k uses the k-th seed pair   */
    int nsplit;          /* "nsplit" photon splitting (ompmc.c:5964)      */
    int precision;       /* omc_precision                                 */
    int nlanes;          /* per-lane schedule: concurrent histories;
                            0 = sized to the GPU                          */
    int stack_depth;     /* per-lane particle stack; 0 = default          */
    int serial;          /* 1 = one lane, one stream: the reference's
                            serial build, history order included          */
    int continue_streams;/* 1 = keep the RANMAR streams where the previous
                            run of this engine left them (same lane count),
                            as successive batches of one reference job;
                            0 = seed them from (ixx, jxx)                  */
    int schedule;        /* omc_schedule                                  */
    long long inflight;  /* wavefront: particles kept in flight, 0 = auto  */
    int chunk_events;    /* wavefront: condensed-history steps a thread
                            takes with one electron before it goes back to
                            the queue; 0 = auto                           */
    int drain_per_warp;  /* wavefront: once every history is injected and
                            fewer than this many particles per 32 threads
                            are in flight (the end-of-run drain), electron
                            interactions run inline and a take follows an
                            electron to the end of its track; 0 = auto,
                            -1 = never                                    */
    int history_stats;   /* wavefront: 1 = also score the history-by-history
                            sums of x and x^2 per region (x = energy one
                            history deposits there), read back with
                            omc_engine_history_sums; 0 = batch sums only
                            (the reference's method)                      */
} omc_run_config;

typedef enum omc_schedule {
    OMC_SCHEDULE_AUTO = 0,      /* wavefront, or per-lane when serial = 1  */
    OMC_SCHEDULE_LANES = 1,     /* each lane transports whole histories in
                                   the reference's stack order             */
    OMC_SCHEDULE_WAVEFRONT = 2  /* photon and electron queues in HBM; one
                                   event per queued particle per iteration */
} omc_schedule;

typedef struct omc_run_stats {
    double ensrc;          /* source kinetic energy, FP64 (score.ensrc)    */
    double transport_ms;   /* device time of the batch loop               */
    long long histories;   /* histories transported                       */
    long long steps;       /* particle events processed                   */
    int max_stack;         /* deepest per-lane stack seen                 */
    int error_flags;       /* OR of device error bits (0 = clean): 1 stack
                              overflow, 2 sampling loop limit, 4 history
                              event limit, 16 queue overflow, 32 grid
                              barrier timeout                              */
    long long voxel_steps; /* geometry steps (howfar calls)               */
    long long deposits;    /* energy deposits (ausgab calls)              */
    double kernel_ms;      /* device time of the transport + batch kernels */
    int warnings;          /* 8: an interpolation index fell outside its
                              table and was clamped to the edge bin (rare
                              rounding at the table ends; the reference
                              reads outside the array there)               */
} omc_run_stats;

omc_status omc_engine_create(int device, omc_engine **out);
void omc_engine_destroy(omc_engine *e);
/* Upload tables (kept resident in FP64 and FP32 layouts). */
omc_status omc_engine_set_tables(omc_engine *e, const omc_tables *t);
/* Upload the voxel geometry and per-region data. */
omc_status omc_engine_set_geometry(omc_engine *e, const omc_phantom *ph,
                                   const omc_regions *r);
omc_status omc_engine_set_source(omc_engine *e, const omc_source *s);

/* Runs nbatch batches of nperbatch histories (replaces omc_dosxyz.c:
 * 1237-1263).  accum_endep/accum_endep2 (host, nreg entries each, may be
 * NULL) receive the sum over batches of the batch energy deposit and of its
 * square, exactly the reference's score.accum_endep/accum_endep2 before
 * accumulateResults(). */
omc_status omc_engine_run(omc_engine *e, const omc_run_config *cfg,
                          double *accum_endep, double *accum_endep2,
                          omc_run_stats *stats);
/* Autotuner of the wavefront run options for the loaded geometry and
 * source: times one-launch runs of sample_histories (2 batches) for every
 * in-flight target of 32, 64, 128 and 192 particles per thread and 1 or 2
 * electron steps per queue take, at cfg's precision and splitting, and
 * writes the fastest into *best (a copy of *cfg with inflight and
 * chunk_events set).  rates (may be NULL) receives the histories/s of the
 * 8 candidates in that order.  The RANMAR streams are left where the last
 * trial ended; seed them for the production run. */
omc_status omc_engine_tune(omc_engine *e, const omc_run_config *cfg,
                           long long sample_histories, omc_run_config *best,
                           double *rates);

/* Same, leaving the tallies on the device; returns device pointers valid
 * until the next run (for resident pipelines and benchmarks). */
omc_status omc_engine_run_resident(omc_engine *e, const omc_run_config *cfg,
                                   const double **d_accum_endep,
                                   const double **d_accum_endep2,
                                   omc_run_stats *stats);

/* History-by-history sums of the last run made with
 * cfg->history_stats = 1 (nreg entries each, may be NULL): sum[r] and
 * sum2[r] over histories of x and x^2, x the energy (MeV) one history
 * deposited in region r, the estimators of Walters, Kawrakow and Rogers,
 * Med. Phys. 29 (2002) 2745: mean = sum/N, variance of the mean =
 * (sum2/N - mean^2)/(N - 1).  *histories = histories merged (N when no
 * error flag is set); *split = histories that touched more regions than
 * the merge table holds (they count as several histories; zero in
 * practice).  The reference has only the batch method (accumEndep,
 * omc_dosxyz.c:696-755), which every run still returns.  History tracking
 * needs a pool of 3 blocks of 384 bytes per particle in flight on the
 * device during the run (14 GB at the FP32 default).  OMC_ERR_STATE if
 * the last run did not track histories. */
omc_status omc_engine_history_sums(omc_engine *e, double *sum, double *sum2,
                                   long long *histories, long long *split);

/* Weighted sums of the batch tallies of the last run: out[b] = sum over
 * regions r of weights[r] * (energy batch b deposited in r), for the
 * nbatch batches of that run (written to *nbatch when not NULL; out holds
 * nbatch doubles).  With weights = dose factor on a region of interest and
 * 0 elsewhere, the spread of out over the batches is the batch uncertainty
 * of the region's mean dose, voxel correlations included.  Available after
 * an omc_engine_run / omc_engine_run_resident whose batches shared one
 * wavefront launch (the default for nbatch > 1); OMC_ERR_STATE otherwise.
 * No counterpart in the reference, which scores per voxel only
 * (accumEndep, omc_dosxyz.c:696-737). */
omc_status omc_engine_batch_sums(omc_engine *e, const double *weights,
                                 double *out, int *nbatch);

/* ------------------------------------------------------------------------
 * Transport that allocates no device memory.  No counterpart in the
 * reference (which has no GPU path).  It is for callers that cannot call
 * cudaMalloc while they run a dose job: applications whose device memory
 * is all handed out by their own pool or caching allocator (a planning
 * system that reserves the GPU at start-up, a framework such as PyTorch
 * that owns the free memory), and services under a fixed device-memory
 * budget, where a new allocation can fail in mid-job or push other work
 * out.  The call itself is synchronous: it returns when the transport has
 * finished, and it reads its counters back to the host.  It is therefore
 * NOT for use inside a CUDA stream capture or a host callback.
 *
 * omc_engine_run_noalloc transports cfg->nperbatch histories (one batch;
 * cfg->nbatch must be 1) on the per-lane schedule with the tables,
 * geometry and source already resident in the engine, and ADDS the energy
 * deposits (MeV, region order, nx*ny*nz+1 doubles) to d_endep, a DEVICE
 * array the caller owns.  All its device work runs on `stream` (a
 * cudaStream_t; NULL is the legacy default stream), after whatever the
 * caller queued there before, so zero d_endep on that same stream (or
 * synchronise first) for a fresh tally.  The RANMAR states, particle
 * stacks and counters live in one file-scope device array of fixed size
 * instead of allocated buffers:
 *   lanes        cfg->nlanes in 1..OMC_NOALLOC_MAX_LANES (0 = the maximum;
 *                cfg->serial = 1 uses one lane, the reference's serial
 *                build)
 *   stack depth  cfg->stack_depth in 1..OMC_NOALLOC_MAX_DEPTH; 0 takes the
 *                depth omc_engine_run takes by default, 48 + 4*nsplit,
 *                which fits only for nsplit <= 4: with stack_depth = 0 a
 *                larger nsplit is refused (pass an explicit depth; a stack
 *                that overflows drops histories and returns OMC_ERR_STACK)
 * which is OMC_NOALLOC_SCRATCH_BYTES (about 19 MiB) on every GPU that
 * loads the library, held until the process exits.  Larger requests are
 * refused with OMC_ERR_ARG.  The first call on a device looks the array's
 * device address up (cudaGetSymbolAddress) with that device current.
 * Every call reuses the same array and leaves its contents behind: the
 * counters are cleared at the start of each call, the streams are
 * re-seeded unless cfg->continue_streams is set (then they continue from
 * the previous no-alloc call with the same lane count).  Calls that
 * overlap on the GPU (several host threads or streams, or several engines
 * on one device) race on the array and must be serialised by the caller.
 * stats may be NULL; its timing fields are host wall time of the call. */
#define OMC_NOALLOC_MAX_LANES 4096
#define OMC_NOALLOC_MAX_DEPTH 64
#define OMC_NOALLOC_SCRATCH_BYTES                                             \
    ((size_t)OMC_NOALLOC_MAX_LANES * (97 + 3) * 4 +                           \
     (size_t)OMC_NOALLOC_MAX_LANES * OMC_NOALLOC_MAX_DEPTH * (8 * 8 + 4) +    \
     (size_t)256)
omc_status omc_engine_run_noalloc(omc_engine *e, const omc_run_config *cfg,
                                  double *d_endep, void *stream,
                                  omc_run_stats *stats);

/* Diagnostics: record, for each iteration of the next wavefront launches
 * (at most `iterations`; 0 switches recording off), the device time in ns
 * and the photons, electrons and histories in flight at its start.
 * omc_engine_trace_read copies the records of the last launch, 4 values
 * each, and their number. */
omc_status omc_engine_trace(omc_engine *e, int iterations);
omc_status omc_engine_trace_read(omc_engine *e, long long *out, int cap, int *n);

/* Free and total device memory of a CUDA device (bytes). */
omc_status omc_device_memory(int device, size_t *free_bytes, size_t *total_bytes);

/* Throughput of scattered FP64 atomicAdd into an array of nreg doubles
 * (atomics/s; ausgab's pattern: every lane of a warp adds to its own
 * voxel), best of 3 launches of 8 blocks x 256 threads per SM, 1024 adds
 * per thread.  The denominator of the transport kernels' tally rate. */
omc_status omc_measure_atomic_rate(int device, long long nreg, double *per_s);

/* RANMAR streams on the device (bit-exact with initRandom/setRandom,
 * omc_random.c:58-187).  Stream k is seeded with the k-th pair of the
 * sequence (ixx, jxx), (ixx, jxx+1), ..., (the reference's per-thread
 * seeding, omc_random.c:72, continued past jxx = 31328 into ixx+1).
 * out[k*n + i] = 24-bit integer of the i-th number of stream k. */
omc_status omc_gpu_ranmar(int device, int ixx, int jxx, int nstreams,
                          long long n, int32_t *out);

/* Seed pair of stream k under the rule above (host helper). */
void omc_stream_seeds(int ixx, int jxx, long long k, int *ixx_k, int *jxx_k);

/* ------------------------------------------------------------------------
 * Dose-influence matrix (omc_matrad).  Replaces the beamlet loop of the
 * matRad front end (ucodes/omc_matrad/omc_matrad.c:1374-1512): for every
 * beamlet, its histories start on the beamlet's bixel, its dose is
 * accumulated separately, converted to Gy per history, thresholded at
 * rel_threshold x the beamlet's maximum and stored as one column of a
 * compressed-sparse-column matrix over voxels x beamlets (equivalently CSR
 * over beamlets x voxels).
 * ---------------------------------------------------------------------- */

/* Beamlet geometry, the fields of matRad's mcSrc structure
 * (omc_matrad.c:543-750): every beamlet is a parallelogram at the
 * isocentre plane, corner + a*side1 + b*side2 with a, b uniform in [0,1),
 * irradiated from the source point of its beam.  All coordinates in cm in
 * the phantom frame. */
typedef struct omc_beamlets {
    int nbeamlets;               /* mcSrc.nBixels                          */
    int nbeams;                  /* entries of the source-point arrays     */
    const int *ibeam;            /* [nbeamlets] beam, 0-based (iBeam - 1)  */
    const double *xsource, *ysource, *zsource; /* [nbeams]                 */
    const double *xcorner, *ycorner, *zcorner; /* [nbeamlets]              */
    const double *xside1, *yside1, *zside1;    /* [nbeamlets]              */
    const double *xside2, *yside2, *zside2;    /* [nbeamlets]              */
} omc_beamlets;

/* Uploads the beamlets; the energy spectrum (or mono energy) and charge
 * still come from omc_engine_set_source.  Requires the geometry. */
omc_status omc_engine_set_beamlets(omc_engine *e, const omc_beamlets *b);

typedef struct omc_dij {
    int nrows;           /* voxels, nx*ny*nz (row = region index - 1)      */
    int ncols;           /* beamlets                                       */
    long long nnz;       /* stored entries                                 */
    long long *col_ptr;  /* [ncols+1] (mxGetJc)                            */
    int *row_idx;        /* [nnz], ascending within a column (mxGetIr)     */
    double *values;      /* [nnz] (mxGetPr); NULL when fp32_values was set */
    float *values_f32;   /* [nnz] when fp32_values was set, else NULL      */
} omc_dij;

void omc_dij_free(omc_dij *d);

typedef struct omc_dij_config {
    double rel_threshold;   /* "relative dose threshold": keep entries
                               strictly above this x the column maximum   */
    const long long *nhist; /* [nbeamlets] histories of each beamlet, or
                               NULL: cfg->nperbatch * cfg->nbatch each
                               (the reference's uniform count)             */
    int fp32_values;        /* 1 = store FP32 values (FP64 accumulation)  */
    long long tally_bytes;  /* device memory for the beamlet tallies that
                               are transported together; 0 = automatic     */
} omc_dij_config;

/* Transports every beamlet's histories and returns the dij in *out (free
 * with omc_dij_free).  Values follow the reference: (sum of the beamlet's
 * energy deposits / nbatch) x 1.602e-10 / (voxel mass x histories of the
 * beamlet), zero where the voxel density is below 0.044 g/cm^3
 * (omc_matrad.c:839-919; the division by nbatch comes from the reference
 * passing the total history count, omc_matrad.c:1418).  cfg->nbatch only
 * enters that normalisation.  With cfg->serial = 1 the beamlets run one
 * after another on one RANMAR stream in the reference's serial order.
 * Beamlets otherwise share one launch: as many beamlet tallies as fit in
 * tally_bytes are resident at once, and histories of different beamlets
 * are in flight together. */
omc_status omc_engine_run_dij(omc_engine *e, const omc_run_config *cfg,
                              const omc_dij_config *dcfg, omc_dij **out,
                              omc_run_stats *stats);

/* ------------------------------------------------------------------------
 * Resident dose jobs.  Several omc_dosxyz-style jobs (own phantom, source,
 * cuts, batches) stay on one engine and share its tables; a round
 * transports the next quota[i] histories of every jobs[i] in ONE launch,
 * their particles in flight together.  History k of a job (counted over
 * rounds) scores in batch k / nperbatch, so a finished job returns the
 * same batch sums as omc_engine_run.  The regions of a job must be built
 * with the engine's tables (same media in the same order).  No
 * counterpart in the reference, which runs one job per process; this is
 * the layer the dose server (omc_server_*) schedules.
 * ---------------------------------------------------------------------- */
typedef struct omc_job omc_job;

/* Device bytes a job of this phantom holds while resident. */
size_t omc_job_device_bytes(const omc_phantom *ph, int nbatch, int precision);

omc_status omc_engine_job_add(omc_engine *e, const omc_phantom *ph,
                              const omc_regions *r, const omc_source *src,
                              long long nperbatch, int nbatch, int precision,
                              omc_job **out);
/* Histories transported so far / in total. */
long long omc_job_done(const omc_job *j);
long long omc_job_histories(const omc_job *j);

/* Beamlet (dij) job resident on the engine: the omc_matrad beamlet loop
 * (ucodes/omc_matrad/omc_matrad.c:1374-1512) as a job that advances in
 * rounds beside field jobs.  History k of the job belongs to beamlet b
 * with sum(nh[0..b-1]) <= k < sum(nh[0..b]) (nh = nhist, or nperbatch *
 * nbatch for every beamlet when nhist is NULL), starts from that beamlet's
 * source (initHistory(ibeamlet), :1084-1254) and scores into the beamlet's
 * own tally; nbatch only divides the dose, as in the reference (:1418).  At
 * most 4096 beamlets per job.  When the job is done,
 * omc_engine_job_dij converts its tallies into the CSC dij that
 * omc_engine_run_dij returns for the same beamlets (values per history,
 * entries above rel_threshold of each beamlet's maximum).  A beamlet job
 * is freed with omc_engine_job_remove.  omc_job_dij_device_bytes is its
 * device footprint. */
omc_status omc_engine_job_add_dij(omc_engine *e, const omc_phantom *ph,
                                  const omc_regions *r, const omc_source *src,
                                  const omc_beamlets *bl,
                                  const long long *nhist, long long nperbatch,
                                  int nbatch, int precision, omc_job **out);
omc_status omc_engine_job_dij(omc_engine *e, omc_job *job,
                              double rel_threshold, int fp32_values,
                              omc_dij **out);
size_t omc_job_dij_device_bytes(const omc_phantom *ph, int nbeamlets,
                                int precision);

/* One launch over njobs jobs of one precision.  cfg supplies nsplit,
 * inflight and the seeds used when the streams are (re)seeded: streams
 * continue between rounds when cfg->continue_streams is set. */
omc_status omc_engine_job_round(omc_engine *e, omc_job *const *jobs,
                                const long long *quota, int njobs,
                                const omc_run_config *cfg,
                                omc_run_stats *stats);
/* Batch sums (score.accum_endep / accum_endep2, nreg entries each, may be
 * NULL) and source energy of the histories transported so far. */
omc_status omc_engine_job_result(omc_engine *e, omc_job *j,
                                 double *accum_endep, double *accum_endep2,
                                 double *ensrc);
void omc_engine_job_remove(omc_engine *e, omc_job *j);

/* ------------------------------------------------------------------------
 * Dose server: continuous batching of dose jobs on one GPU.  Jobs are
 * submitted from any thread and queue in arrival order; an admission
 * thread moves the head job onto the device (phantom, source, tallies) as
 * soon as the device-memory budget and the job limit allow, overlapping
 * its upload with transport; a scheduler thread runs rounds: one launch in
 * which every resident job advances by its share of round_histories
 * histories, so jobs that arrive while others run join at the next round
 * and small jobs finish without waiting for large ones.  Finished jobs
 * leave the device at once.  No counterpart in the reference.
 * ---------------------------------------------------------------------- */
typedef struct omc_server omc_server;

typedef struct omc_server_config {
    int device;
    int precision;              /* OMC_FP32 or OMC_FP64, for every job     */
    long long hbm_budget;       /* device bytes for resident jobs; 0 = half
                                   the free memory at creation            */
    int max_jobs;               /* resident jobs at most; 0 = 256          */
    long long round_histories;  /* histories per round over all resident
                                   jobs; 0 = adaptive: 4e6 while more than
                                   two jobs are resident, else a quarter of
                                   their histories left, at most 4x the
                                   shortest job's, within [4e6, 3.2e7]     */
    int nsplit;                 /* photon splitting, every job (0 = 1)     */
    int ixx, jxx;               /* RANMAR seeds of the server's streams    */
    int policy;                 /* round quotas: OMC_SERVE_SHORTEST_FIRST
                                   (fill the round with the jobs that have
                                   the fewest histories left; default) or
                                   OMC_SERVE_EQUAL_SHARES                  */
} omc_server_config;

enum { OMC_SERVE_SHORTEST_FIRST = 0, OMC_SERVE_EQUAL_SHARES = 1 };

/* The server's media: every job's phantom media must be among them.
 * data_keys supplies "pegs file", "pgs4form file" and "data folder"; the
 * tables are built once and stay resident. */
omc_status omc_server_create(const omc_server_config *cfg,
                             const omc_input *data_keys, int nmed,
                             const char *const *media, omc_server **out);

typedef struct omc_server_job {
    const omc_phantom *phantom; /* copied by submit                        */
    const omc_source *source;   /* copied by submit                        */
    double ecut, pcut;          /* "global ecut" / "global pcut" (MeV)     */
    long long nperbatch;
    int nbatch;
} omc_server_job;

omc_status omc_server_submit(omc_server *s, const omc_server_job *job,
                             long long *id);

typedef struct omc_server_result {
    double ensrc;               /* source kinetic energy (MeV)             */
    long long histories;
    double submit_s;            /* times since omc_server_create (s)       */
    double admit_s;             /* resident on the device                  */
    double finish_s;            /* tallies back on the host                */
    int rounds;                 /* rounds the job took part in             */
    int status;                 /* omc_status of the job                   */
} omc_server_result;

/* Waits for job id (timeout_s < 0: without limit; OMC_ERR_LIMIT on
 * timeout, the job stays queued), copies its batch sums (nreg entries
 * each, may be NULL) and forgets the job. */
omc_status omc_server_wait(omc_server *s, long long id, double timeout_s,
                           double *accum_endep, double *accum_endep2,
                           omc_server_result *res);

/* A beamlet job: the dose-influence matrix of bl on job's phantom, as
 * omc_engine_run_dij computes it, i.e. the beamlet loop of the matRad front
 * end (ucodes/omc_matrad/omc_matrad.c:1374-1512) queued on the server
 * beside field jobs (job->source gives the spectrum and
 * charge; its geometry is the beamlets').  nhist[i] histories for beamlet
 * i, or job->nperbatch * job->nbatch each when nhist is NULL; job->nbatch
 * batches; at most 4096 beamlets.  All inputs are copied.  The job is
 * admitted and scheduled like a field job (omc_engine_job_add_dij): it is
 * resident with one tally per beamlet, advances in the same rounds (its
 * histories share launches with the other jobs' histories), and is turned
 * into its CSC dij on the device when its last history is done. */
omc_status omc_server_submit_dij(omc_server *s, const omc_server_job *job,
                                 const omc_beamlets *bl,
                                 const long long *nhist, double rel_threshold,
                                 int fp32_values, long long *id);

/* Waits for beamlet job id as omc_server_wait does and hands over its dij
 * (*out, freed with omc_dij_free); res->histories = all its histories. */
omc_status omc_server_wait_dij(omc_server *s, long long id, double timeout_s,
                               omc_dij **out, omc_server_result *res);

typedef struct omc_server_stats {
    long long submitted, finished, rounds, histories;
    int max_resident;           /* most jobs resident at once              */
    int max_round_jobs;         /* most jobs in one round                  */
    long long max_resident_bytes;
    double transport_s;         /* device time of all rounds               */
} omc_server_stats;

omc_status omc_server_get_stats(omc_server *s, omc_server_stats *st);
/* Histories of the next round, as the scheduler picks them: `configured`
 * (round_histories) when > 0; else the adaptive size from the resident
 * jobs' histories left (`backlog`), the fewest any of them has left
 * (`shortest`) and their number (`resident`).  Host only. */
long long omc_server_round_histories(long long configured, long long backlog, long long shortest,
                                     int resident);
/* Stops both threads after the current round; queued jobs are dropped. */
void omc_server_destroy(omc_server *s);

/* ------------------------------------------------------------------------
 * matRad entry point.  Replaces mexFunction of the omc_matrad front end
 * (omc_matrad.c:1258-1530): the same five inputs as plain C data, the same
 * sparse dij out.  A MATLAB binding wraps it in a few lines (mxGetPr of
 * each field in, mxCreateSparse + copy out).
 * ---------------------------------------------------------------------- */
typedef struct omc_matrad_geo {
    int nx, ny, nz;              /* size of cubeRho (x fastest)            */
    const double *cube_rho;      /* cubeRho, [nx*ny*nz] g/cm^3             */
    const int *cube_mat_ix;      /* cubeMatIx (int32), 1-based material    */
    int nmaterials;              /* entries of mcGeo.material              */
    const char *const *materials;/* mcGeo.material (pegs4 medium names)    */
    const double *xbounds, *ybounds, *zbounds; /* mcGeo.x/y/zBounds (cm)   */
} omc_matrad_geo;

typedef struct omc_matrad_opt {  /* mcOpt (omc_matrad.c:62-250)            */
    long long n_histories;       /* nHistories: histories per beamlet      */
    int n_batches;               /* nBatches                               */
    int n_split;                 /* nSplit                                 */
    const char *spectrum_file;   /* spectrumFile; NULL or "" = monoEnergy
                                    (the reference always reads a file)    */
    double mono_energy;          /* monoEnergy (MeV)                       */
    int charge;                  /* charge: read but not applied, the
                                    reference's beams are always photons   */
    double global_ecut, global_pcut;
    int random_seeds[2];         /* randomSeeds                            */
    const char *pegs_file, *pgs4form_file, *data_folder, *output_folder;
    double rel_dose_threshold;   /* relDoseThreshold                       */
    int verbose;                 /* verbose: progress lines on stdout      */
} omc_matrad_opt;

/* Builds tables, regions and source from the inputs, transports every
 * beamlet on `device` (precision OMC_FP64 or OMC_FP32; serial = 1 runs the
 * reference's serial order) and returns the dij in *out (free with
 * omc_dij_free). */
omc_status omc_matrad_dij(int device, const omc_matrad_geo *geo,
                          const omc_beamlets *src, const omc_matrad_opt *opt,
                          int precision, int serial, omc_dij **out);

#ifdef __cplusplus
}
#endif
#endif /* OMC_GPU_H */
