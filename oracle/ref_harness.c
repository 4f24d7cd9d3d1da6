/*
 * Test-infrastructure harness around the UNMODIFIED reference (edoerner/ompMC).
 *
 * This file is part of the oracle: it is compiled only by oracle/Makefile,
 * against the reference sources where they lie (REF/src, REF/ucodes), into
 * oracle/_ref/.  Nothing in the product links or runs it.  It exposes the
 * reference's own code paths as small sub-commands whose raw outputs pin the
 * product's table builders and the oracle's transport restatement:
 *
 *   rng    <ixx> <jxx> <n> <out>   RANMAR stream (omc_random.c:58-187) as int32
 *                                  values v, number = v * 2^-24
 *   tables <input-without-.inp> <out>
 *                                  initPhantom/initMediaData/initSource/
 *                                  initRegions/initVrt (omc_dosxyz.c:1167-1179)
 *                                  and a dump of every table they build
 *   dose   <input-without-.inp> <out> [nthreads]
 *                                  the batch/history loop of omc_dosxyz
 *                                  (omc_dosxyz.c:1237-1263) with a dump of the
 *                                  raw per-voxel batch sums before
 *                                  accumulateResults() rescales them
 *
 * The omc_dosxyz user code is pulled in by #include from the reference tree
 * with its main() renamed, so its geometry/source/scoring globals and
 * callbacks (howfar, hownear, ausgab, initHistory) are the reference's own.
 */
#define main ref_dosxyz_main
#include "omc_dosxyz.c"
#undef main

#include <stdint.h>

/* ---- dump format: "OMCT" then records {u32 len, name, u8 type, u64 n, data} */
static FILE *dump_open(const char *path) {
    FILE *f = fopen(path, "wb");
    if (!f) { fprintf(stderr, "cannot open %s\n", path); exit(2); }
    fwrite("OMCT", 1, 4, f);
    return f;
}
static void dump_arr(FILE *f, const char *name, char type, const void *p,
                     uint64_t n) {
    uint32_t len = (uint32_t)strlen(name);
    fwrite(&len, 4, 1, f);
    fwrite(name, 1, len, f);
    fwrite(&type, 1, 1, f);
    fwrite(&n, 8, 1, f);
    size_t esz = (type == 'd') ? 8 : 4;
    if (n) fwrite(p, esz, n, f);
}
static void dump_d(FILE *f, const char *name, const double *p, uint64_t n) {
    dump_arr(f, name, 'd', p, n);
}
static void dump_i(FILE *f, const char *name, const int *p, uint64_t n) {
    dump_arr(f, name, 'i', p, n);
}
static void dump_scalar(FILE *f, const char *name, double v) {
    dump_arr(f, name, 'd', &v, 1);
}

static void set_item(const char *key, const char *value) {
    strcpy(input_items[input_idx].key, key);
    strcpy(input_items[input_idx].value, value);
    input_idx++;
}

static int cmd_rng(int ixx, int jxx, long n, const char *out) {
    char buf[64];
    snprintf(buf, sizeof buf, "%d %d", ixx, jxx);
    input_idx = 0;
    set_item("rng seeds", buf);
    initRandom();
    int *vals = malloc(n * sizeof(int));
    for (long i = 0; i < n; i++) {
        double r = setRandom();
        vals[i] = (int)(r * 16777216.0);
    }
    FILE *f = dump_open(out);
    dump_i(f, "rng", vals, (uint64_t)n);
    fclose(f);
    free(vals);
    cleanRandom();
    return 0;
}

static void init_all(char *input) {
    parseInputFile(input);
    initPhantom();
    initMediaData();
    initSource();
    initRegions();
    initVrt();
    initScore();
}

static void dump_tables(const char *out) {
    int nmed = media.nmed;
    FILE *f = dump_open(out);
    dump_scalar(f, "nmed", nmed);
    /* pegs scalars */
    double tmp[MXMED];
#define PEGS_D(field) \
    for (int i = 0; i < nmed; i++) tmp[i] = pegs_data.field[i]; \
    dump_d(f, "pegs." #field, tmp, nmed);
    PEGS_D(rho) PEGS_D(rlc) PEGS_D(ae) PEGS_D(ap) PEGS_D(ue) PEGS_D(up)
    PEGS_D(te) PEGS_D(thmoll) PEGS_D(delcm)
    int itmp[MXMED];
    for (int i = 0; i < nmed; i++) itmp[i] = pegs_data.meke[i];
    dump_i(f, "pegs.meke", itmp, nmed);
    for (int i = 0; i < nmed; i++) itmp[i] = pegs_data.ne[i];
    dump_i(f, "pegs.ne", itmp, nmed);
    /* photon */
    dump_d(f, "photon.ge0", photon_data.ge0, nmed);
    dump_d(f, "photon.ge1", photon_data.ge1, nmed);
    uint64_t ng = (uint64_t)nmed * MXGE;
    dump_d(f, "photon.gmfp0", photon_data.gmfp0, ng);
    dump_d(f, "photon.gmfp1", photon_data.gmfp1, ng);
    dump_d(f, "photon.gbr10", photon_data.gbr10, ng);
    dump_d(f, "photon.gbr11", photon_data.gbr11, ng);
    dump_d(f, "photon.gbr20", photon_data.gbr20, ng);
    dump_d(f, "photon.gbr21", photon_data.gbr21, ng);
    dump_d(f, "photon.cohe0", photon_data.cohe0, ng);
    dump_d(f, "photon.cohe1", photon_data.cohe1, ng);
    /* rayleigh */
    uint64_t nr = (uint64_t)nmed * MXRAYFF;
    dump_d(f, "rayleigh.xgrid", rayleigh_data.xgrid, nr);
    dump_d(f, "rayleigh.fcum", rayleigh_data.fcum, nr);
    dump_d(f, "rayleigh.b_array", rayleigh_data.b_array, nr);
    dump_d(f, "rayleigh.c_array", rayleigh_data.c_array, nr);
    dump_i(f, "rayleigh.i_array", rayleigh_data.i_array, nr);
    dump_d(f, "rayleigh.pmax0", rayleigh_data.pmax0, ng);
    dump_d(f, "rayleigh.pmax1", rayleigh_data.pmax1, ng);
    /* pair */
    dump_d(f, "pair.dl1", pair_data.dl1, nmed * 8);
    dump_d(f, "pair.dl2", pair_data.dl2, nmed * 8);
    dump_d(f, "pair.dl3", pair_data.dl3, nmed * 8);
    dump_d(f, "pair.dl4", pair_data.dl4, nmed * 8);
    dump_d(f, "pair.dl5", pair_data.dl5, nmed * 8);
    dump_d(f, "pair.dl6", pair_data.dl6, nmed * 8);
    dump_d(f, "pair.bpar0", pair_data.bpar0, nmed);
    dump_d(f, "pair.bpar1", pair_data.bpar1, nmed);
    dump_d(f, "pair.delcm", pair_data.delcm, nmed);
    dump_d(f, "pair.zbrang", pair_data.zbrang, nmed);
    /* electron */
    uint64_t ne = (uint64_t)nmed * MXEKE;
#define ELEC(field) dump_d(f, "electron." #field, electron_data.field, ne);
    ELEC(esig0) ELEC(esig1) ELEC(psig0) ELEC(psig1)
    ELEC(ededx0) ELEC(ededx1) ELEC(pdedx0) ELEC(pdedx1)
    ELEC(ebr10) ELEC(ebr11) ELEC(pbr10) ELEC(pbr11) ELEC(pbr20) ELEC(pbr21)
    ELEC(tmxs0) ELEC(tmxs1) ELEC(blcce0) ELEC(blcce1)
    ELEC(etae_ms0) ELEC(etae_ms1) ELEC(etap_ms0) ELEC(etap_ms1)
    ELEC(q1ce_ms0) ELEC(q1ce_ms1) ELEC(q1cp_ms0) ELEC(q1cp_ms1)
    ELEC(q2ce_ms0) ELEC(q2ce_ms1) ELEC(q2cp_ms0) ELEC(q2cp_ms1)
    ELEC(e_array)
    dump_d(f, "electron.range_ep", electron_data.range_ep, 2 * ne);
    dump_d(f, "electron.eke0", electron_data.eke0, nmed);
    dump_d(f, "electron.eke1", electron_data.eke1, nmed);
    dump_i(f, "electron.sig_ismonotone", electron_data.sig_ismonotone,
           2 * nmed);
    dump_d(f, "electron.esig_e", electron_data.esig_e, nmed);
    dump_d(f, "electron.psig_e", electron_data.psig_e, nmed);
    dump_d(f, "electron.xcc", electron_data.xcc, nmed);
    dump_d(f, "electron.blcc", electron_data.blcc, nmed);
    dump_d(f, "electron.expeke1", electron_data.expeke1, nmed);
    /* spin */
    dump_scalar(f, "spin.b2spin_min", spin_data.b2spin_min);
    dump_scalar(f, "spin.dbeta2i", spin_data.dbeta2i);
    dump_scalar(f, "spin.espml", spin_data.espml);
    dump_scalar(f, "spin.dleneri", spin_data.dleneri);
    dump_scalar(f, "spin.dqq1i", spin_data.dqq1i);
    dump_d(f, "spin.spin_rej", spin_data.spin_rej,
           (uint64_t)nmed * 2 * (MXE_SPIN1 + 1) * (MXQ_SPIN + 1) *
               (MXU_SPIN + 1));
    /* mscat */
    uint64_t nm = (uint64_t)(MXL_MS + 1) * (MXQ_MS + 1) * (MXU_MS + 1);
    dump_d(f, "mscat.ums", mscat_data.ums_array, nm);
    dump_d(f, "mscat.fms", mscat_data.fms_array, nm);
    /* the last u entry of wms/ims is never read (omc ompmc.c:3250-3257) */
    {
        double *w = malloc(nm * sizeof(double));
        int *m = malloc(nm * sizeof(int));
        for (uint64_t i = 0; i < nm; i++) {
            int last = (int)(i % (MXU_MS + 1)) == MXU_MS;
            w[i] = last ? 0.0 : mscat_data.wms_array[i];
            m[i] = last ? 0 : mscat_data.ims_array[i];
        }
        dump_d(f, "mscat.wms", w, nm);
        dump_i(f, "mscat.ims", m, nm);
        free(w);
        free(m);
    }
    dump_scalar(f, "mscat.dllambi", mscat_data.dllambi);
    dump_scalar(f, "mscat.dqmsi", mscat_data.dqmsi);
    /* regions, source */
    int nreg = geometry.isize * geometry.jsize * geometry.ksize + 1;
    dump_i(f, "region.med", region.med, nreg);
    dump_d(f, "region.rhof", region.rhof, nreg);
    dump_d(f, "region.pcut", region.pcut, nreg);
    dump_d(f, "region.ecut", region.ecut, nreg);
    if (source.spectrum) {
        dump_d(f, "source.cdfinv1", source.cdfinv1, (int)source.deltak);
        dump_d(f, "source.cdfinv2", source.cdfinv2, (int)source.deltak);
    }
    double sg[8] = {source.xinl, source.xinu, source.yinl, source.yinu,
                    source.xsize, source.ysize, source.ixinl, source.ixinu};
    dump_d(f, "source.geom", sg, 8);
    double sg2[2] = {source.iyinl, source.iyinu};
    dump_d(f, "source.iy", sg2, 2);
    fclose(f);
}

static int cmd_tables(char *input, const char *out) {
    init_all(input);
    dump_tables(out);
    return 0;
}

static int cmd_dose(char *input, const char *out, int nthreads) {
    init_all(input);
#ifdef _OPENMP
    if (nthreads <= 0) nthreads = omp_get_num_procs();
    omp_set_num_threads(nthreads);
#else
    nthreads = 1;
#endif
    #pragma omp parallel
    {
        initRandom();
        initStack();
    }
    char buffer[BUFFER_SIZE];
    getInputValue(buffer, "ncase");
    int nhist = atoi(buffer);
    getInputValue(buffer, "nbatch");
    int nbatch = atoi(buffer);
    if (nhist / nbatch == 0) nhist = nbatch;
    int nperbatch = nhist / nbatch;
    int gridsize = geometry.isize * geometry.jsize * geometry.ksize;

    double t0 = omc_get_time();
    for (int ibatch = 0; ibatch < nbatch; ibatch++) {
        int ihist;
        #pragma omp parallel for schedule(dynamic)
        for (ihist = 0; ihist < nperbatch; ihist++) {
            initHistory();
            shower();
        }
        accumEndep();
    }
    double t1 = omc_get_time();

    FILE *f = dump_open(out);
    dump_d(f, "accum_endep", score.accum_endep, gridsize + 1);
    dump_d(f, "accum_endep2", score.accum_endep2, gridsize + 1);
    dump_scalar(f, "ensrc", score.ensrc);
    dump_scalar(f, "nperbatch", nperbatch);
    dump_scalar(f, "nbatch", nbatch);
    dump_scalar(f, "transport_seconds", t1 - t0);
    dump_scalar(f, "nthreads", nthreads);
    fclose(f);
    return 0;
}

int main(int argc, char **argv) {
    if (argc >= 6 && strcmp(argv[1], "rng") == 0)
        return cmd_rng(atoi(argv[2]), atoi(argv[3]), atol(argv[4]), argv[5]);
    if (argc >= 4 && strcmp(argv[1], "tables") == 0)
        return cmd_tables(argv[2], argv[3]);
    if (argc >= 4 && strcmp(argv[1], "dose") == 0)
        return cmd_dose(argv[2], argv[3], argc >= 5 ? atoi(argv[4]) : 0);
    fprintf(stderr,
            "usage: ref_harness rng IXX JXX N OUT | tables INP OUT | "
            "dose INP OUT [NTHREADS]\n");
    return 2;
}
