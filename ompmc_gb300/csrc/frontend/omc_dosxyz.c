/* omc_dosxyz: the command-line dose calculation of ompMC on the GB300
 * engine.
 *
 * Same command line and .inp file as the reference front end
 * (ucodes/omc_dosxyz/omc_dosxyz.c:1075-1300):
 *
 *   omc_dosxyz -i <input without .inp> -o <output name> [--verbose]
 *
 * reads "phantom file", "pegs file", "pgs4form file", "data folder",
 * "spectrum file" or "mono energy", "charge", "ssd", "collimator bounds",
 * "global ecut", "global pcut", "rng seeds", "nsplit", "ncase", "nbatch"
 * and "output folder", transports ncase histories in nbatch batches and
 * writes <output folder><output name>.3ddose (mean dose per history and
 * batch relative uncertainty, normalised by the histories per batch as the
 * reference does, omc_dosxyz.c:1282).
 *
 * The per-thread OpenMP history loop (omc_dosxyz.c:1237-1263) becomes one
 * omc_engine_run call.  Options beyond the reference's:
 *   --fp32 | --fp64        transport arithmetic (default FP64, the
 *                          reference's; tallies are FP64 either way)
 *   --serial               one RANMAR stream, histories in order: the
 *                          reference's serial build, history by history
 *   --device <n>           CUDA device (default 0)
 * Exit status is EXIT_FAILURE with a message on any error, as in the
 * reference. */

#include <ctype.h>
#include <getopt.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>

#include "omc_gpu.h"

static double now_s(void) {
    struct timespec ts;
    clock_gettime(CLOCK_MONOTONIC, &ts);
    return (double)ts.tv_sec + 1e-9 * (double)ts.tv_nsec;
}

static void die(const char *what, omc_status s) {
    fprintf(stderr, "%s: %s (%s)\n", what, omc_last_error(), omc_status_string(s));
    exit(EXIT_FAILURE);
}

#define CHECK(call)                                  \
    do {                                             \
        omc_status s_ = (call);                      \
        if (s_ != OMC_OK) die(#call, s_);            \
    } while (0)

/* Key value with every blank removed (the reference's removeSpaces). */
static int get_compact(const omc_input *in, const char *key, char *dest, size_t cap) {
    char raw[1024];
    if (omc_input_get(in, key, raw, sizeof raw) != 1) return 0;
    size_t n = 0;
    for (const char *p = raw; *p && n + 1 < cap; ++p)
        if (!isspace((unsigned char)*p)) dest[n++] = *p;
    dest[n] = '\0';
    return 1;
}

static long long get_int(const omc_input *in, const char *key, int required, long long dflt) {
    char buf[256];
    if (omc_input_get(in, key, buf, sizeof buf) != 1) {
        if (required) {
            fprintf(stderr, "Can not find '%s' key on input file.\n", key);
            exit(EXIT_FAILURE);
        }
        return dflt;
    }
    return atoll(buf);
}

int main(int argc, char **argv) {
    double tbegin = now_s();
    int verbose = 0, serial = 0, precision = OMC_FP64, device = 0;
    const char *input_file = NULL, *output_file = NULL;
    enum { OPT_FP32 = 256, OPT_FP64, OPT_SERIAL, OPT_DEVICE };
    static struct option opts[] = {
        {"verbose", no_argument, 0, 'v'},  {"brief", no_argument, 0, 'b'},
        {"input", required_argument, 0, 'i'}, {"output", required_argument, 0, 'o'},
        {"fp32", no_argument, 0, OPT_FP32}, {"fp64", no_argument, 0, OPT_FP64},
        {"serial", no_argument, 0, OPT_SERIAL}, {"device", required_argument, 0, OPT_DEVICE},
        {0, 0, 0, 0}};
    for (;;) {
        int c = getopt_long(argc, argv, "i:o:", opts, NULL);
        if (c == -1) break;
        switch (c) {
            case 'v': verbose = 1; break;
            case 'b': verbose = 0; break;
            case 'i': input_file = optarg; break;
            case 'o': output_file = optarg; break;
            case OPT_FP32: precision = OMC_FP32; break;
            case OPT_FP64: precision = OMC_FP64; break;
            case OPT_SERIAL: serial = 1; break;
            case OPT_DEVICE: device = atoi(optarg); break;
            default: exit(EXIT_FAILURE);
        }
    }
    if (!input_file || !output_file) {
        fprintf(stderr, "usage: %s -i <input without .inp> -o <output name> [--verbose] "
                        "[--fp32|--fp64] [--serial] [--device n]\n", argv[0]);
        return EXIT_FAILURE;
    }

    omc_input *in = NULL;
    CHECK(omc_input_parse(input_file, &in));

    char path[1024];
    if (!get_compact(in, "phantom file", path, sizeof path)) {
        fprintf(stderr, "Can not find 'phantom file' key on input file.\n");
        return EXIT_FAILURE;
    }
    omc_phantom *ph = NULL;
    CHECK(omc_phantom_read(path, &ph));
    omc_tables *tab = NULL;
    CHECK(omc_tables_build(in, ph->nmed, (const char(*)[OMC_NAME_LEN])ph->med_names, &tab));
    omc_source *src = NULL;
    CHECK(omc_source_build(in, ph, &src));
    omc_regions *reg = NULL;
    CHECK(omc_regions_build(in, ph, tab, &reg));

    long long nhist = get_int(in, "ncase", 1, 0);
    int nbatch = (int)get_int(in, "nbatch", 1, 0);
    if (nbatch <= 0) {
        fprintf(stderr, "'nbatch' must be positive.\n");
        return EXIT_FAILURE;
    }
    if (nbatch < 2) {  /* accumulateResults divides by nbatch - 1 (omc_dosxyz.c:747) */
        fprintf(stderr, "'nbatch' must be at least 2: the batch uncertainty divides by nbatch - 1.\n");
        return EXIT_FAILURE;
    }
    if (nhist / nbatch == 0) nhist = nbatch;
    long long nperbatch = nhist / nbatch;
    nhist = nperbatch * nbatch;

    char seeds[256];
    int ixx = 97, jxx = 33;
    if (omc_input_get(in, "rng seeds", seeds, sizeof seeds) == 1 && sscanf(seeds, "%d %d", &ixx, &jxx) != 2) {
        fprintf(stderr, "'rng seeds' needs two integers.\n");
        return EXIT_FAILURE;
    }
    int nsplit = (int)get_int(in, "nsplit", 0, 1);

    omc_engine *eng = NULL;
    CHECK(omc_engine_create(device, &eng));
    CHECK(omc_engine_set_tables(eng, tab));
    CHECK(omc_engine_set_geometry(eng, ph, reg));
    CHECK(omc_engine_set_source(eng, src));

    printf("Total number of particle histories: %lld\n", nhist);
    printf("Number of statistical batches: %d\n", nbatch);
    printf("Histories per batch: %lld\n", nperbatch);
    printf("Execution time up to this point : %8.2f seconds\n", now_s() - tbegin);

    int nreg = ph->nx * ph->ny * ph->nz + 1;
    double *acc = calloc((size_t)nreg, sizeof(double));
    double *acc2 = calloc((size_t)nreg, sizeof(double));
    double *dose = calloc((size_t)nreg, sizeof(double));
    double *unc = calloc((size_t)nreg, sizeof(double));
    if (!acc || !acc2 || !dose || !unc) {
        fprintf(stderr, "out of host memory\n");
        return EXIT_FAILURE;
    }
    omc_run_config cfg;
    memset(&cfg, 0, sizeof cfg);
    cfg.nperbatch = nperbatch;
    cfg.nbatch = nbatch;
    cfg.ixx = ixx;
    cfg.jxx = jxx;
    cfg.nsplit = nsplit;
    cfg.precision = precision;
    cfg.serial = serial;
    cfg.schedule = OMC_SCHEDULE_AUTO;
    omc_run_stats st;
    CHECK(omc_engine_run(eng, &cfg, acc, acc2, &st));

    printf("Simulation finished\n");
    printf("Execution time up to this point : %8.2f seconds\n", now_s() - tbegin);
    printf("Transport: %.3f s on the GPU, %.4g histories/s (%s)\n", st.transport_ms * 1e-3,
           st.transport_ms > 0 ? (double)nhist / (st.transport_ms * 1e-3) : 0.0,
           precision == OMC_FP32 ? "FP32 transport, FP64 tallies" : "FP64");
    if (verbose) {
        double etot = 0.0;
        for (int i = 1; i < nreg; ++i) etot += acc[i];
        printf("Fraction of incident energy deposited in the phantom: %5.4f\n", etot / st.ensrc);
    }

    char folder[1024];
    if (!get_compact(in, "output folder", folder, sizeof folder)) {
        fprintf(stderr, "Can not find 'output folder' key on input file.\n");
        return EXIT_FAILURE;
    }
    if (verbose) {
        char tpath[2200];
        snprintf(tpath, sizeof tpath, "%s%s.omct", folder, output_file);
        CHECK(omc_tables_dump(tab, tpath));
    }
    CHECK(omc_accumulate_results(ph, acc, acc2, 1, nperbatch, nbatch, dose, unc));
    char out[2200];
    snprintf(out, sizeof out, "%s%s.3ddose", folder, output_file);
    CHECK(omc_write_3ddose(out, ph, dose, unc));

    omc_engine_destroy(eng);
    omc_regions_free(reg);
    omc_source_free(src);
    omc_tables_free(tab);
    omc_phantom_free(ph);
    omc_input_free(in);
    free(acc);
    free(acc2);
    free(dose);
    free(unc);
    printf("Total execution time : %8.5f seconds\n", now_s() - tbegin);
    return EXIT_SUCCESS;
}
