/*
 * Runs the reference's omc_matrad front end (mexFunction, compiled
 * unmodified from its own source) outside MATLAB.  TEST INFRASTRUCTURE
 * ONLY: it pins the oracle's beamlet path and dose-influence matrix.
 *
 *   matrad_harness <dir>
 *
 * reads the five mexFunction inputs from <dir> (written by
 * oracle/binding.py: cubeRho and cubeMatIx as raw arrays, mcGeo, mcSrc
 * and mcOpt as text) and writes the returned sparse matrix to
 * <dir>/dij.bin: int64 nrows, ncols, nnz; int64 jc[ncols+1];
 * int64 ir[nnz]; float64 pr[nnz].
 *
 * The MEX API here is a small stand-in: numeric arrays, structs with named
 * fields, cells of strings, a sparse matrix, num2str, and no-op waitbar /
 * close calls.  mxRealloc never shrinks a block, as MATLAB's allocator
 * leaves a shrunk block in place (the front end shrinks its row-index
 * array with the size of an int).
 */
#include <stdarg.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "mex.h"

enum kind { K_DOUBLE, K_INT32, K_LOGICAL, K_CHAR, K_STRUCT, K_CELL, K_SPARSE };

struct mxArray_tag {
    enum kind kind;
    mwSize ndim;
    mwSize dims[3];
    void *data;  /* doubles, int32, logicals, chars; cells: mxArray*[] */
    int nfields; /* struct: one element */
    char **names;
    mxArray **fields;
    mwIndex *ir, *jc; /* sparse */
    mwSize nzmax;
};

/* Blocks with their size in front, so mxRealloc knows the old size. */
static void *blk_alloc(size_t n) {
    size_t *p = malloc(sizeof(size_t) * 2 + (n ? n : 1));
    if (!p) {
        fprintf(stderr, "harness: out of memory\n");
        exit(3);
    }
    p[0] = n;
    return p + 2;
}
static size_t blk_size(void *q) { return ((size_t *)q)[-2]; }
static void blk_free(void *q) {
    if (q) free((size_t *)q - 2);
}

void *mxRealloc(void *q, mwSize n) {
    if (!q) return blk_alloc(n);
    if (n <= blk_size(q)) return q;
    void *r = blk_alloc(n);
    memcpy(r, q, blk_size(q));
    blk_free(q);
    return r;
}

static mxArray *new_array(enum kind k) {
    mxArray *a = calloc(1, sizeof(mxArray));
    a->kind = k;
    a->ndim = 2;
    a->dims[0] = a->dims[1] = 1;
    a->dims[2] = 1;
    return a;
}

static mxArray *new_doubles(size_t n, const double *v) {
    mxArray *a = new_array(K_DOUBLE);
    a->dims[0] = 1;
    a->dims[1] = n;
    a->data = blk_alloc(n * sizeof(double));
    if (v) memcpy(a->data, v, n * sizeof(double));
    return a;
}

mxArray *mxCreateDoubleScalar(double v) { return new_doubles(1, &v); }

mxArray *mxCreateString(const char *s) {
    mxArray *a = new_array(K_CHAR);
    a->dims[1] = strlen(s);
    a->data = blk_alloc(strlen(s) + 1);
    strcpy(a->data, s);
    return a;
}

mxArray *mxCreateSparse(mwSize m, mwSize n, mwSize nzmax, mxComplexity c) {
    (void)c;
    mxArray *a = new_array(K_SPARSE);
    a->dims[0] = m;
    a->dims[1] = n;
    a->nzmax = nzmax ? nzmax : 1;
    a->data = blk_alloc(a->nzmax * sizeof(double));
    a->ir = blk_alloc(a->nzmax * sizeof(mwIndex));
    a->jc = blk_alloc((n + 1) * sizeof(mwIndex));
    memset(a->jc, 0, (n + 1) * sizeof(mwIndex));
    return a;
}

void mxDestroyArray(mxArray *a) {
    if (!a) return;
    if (a->kind == K_STRUCT) {
        for (int i = 0; i < a->nfields; i++) {
            free(a->names[i]);
            mxDestroyArray(a->fields[i]);
        }
        free(a->names);
        free(a->fields);
    } else if (a->kind == K_CELL) {
        mxArray **c = a->data;
        for (mwSize i = 0; i < a->dims[0] * a->dims[1]; i++) mxDestroyArray(c[i]);
    }
    if (a->kind == K_SPARSE) {
        blk_free(a->ir);
        blk_free(a->jc);
    }
    blk_free(a->data);
    free(a);
}

mxArray *mxGetField(const mxArray *a, mwIndex i, const char *name) {
    (void)i;
    if (!a || a->kind != K_STRUCT) return NULL;
    for (int k = 0; k < a->nfields; k++)
        if (strcmp(a->names[k], name) == 0) return a->fields[k];
    fprintf(stderr, "harness: struct field '%s' missing\n", name);
    exit(3);
}
int mxGetNumberOfFields(const mxArray *a) { return a->nfields; }
double *mxGetPr(const mxArray *a) { return (double *)a->data; }
double mxGetScalar(const mxArray *a) {
    if (a->kind == K_INT32) return (double)((int32_t *)a->data)[0];
    return ((double *)a->data)[0];
}
mxLogical *mxGetLogicals(const mxArray *a) { return (mxLogical *)a->data; }
const mwSize *mxGetDimensions(const mxArray *a) { return a->dims; }
mwSize mxGetNumberOfDimensions(const mxArray *a) { return a->ndim; }
bool mxIsDouble(const mxArray *a) { return a->kind == K_DOUBLE; }
bool mxIsInt32(const mxArray *a) { return a->kind == K_INT32; }
bool mxIsStruct(const mxArray *a) { return a->kind == K_STRUCT; }
mxArray *mxGetCell(const mxArray *a, mwIndex i) { return ((mxArray **)a->data)[i]; }
mwIndex mxCalcSingleSubscript(const mxArray *a, mwSize nsubs, const mwIndex *subs) {
    mwIndex idx = 0, mul = 1;
    for (mwSize k = 0; k < nsubs; k++) {
        idx += subs[k] * mul;
        mul *= a->dims[k];
    }
    return idx;
}
char *mxArrayToString(const mxArray *a) {
    if (!a || a->kind != K_CHAR) return NULL;
    char *s = malloc(strlen(a->data) + 1);
    strcpy(s, a->data);
    return s;
}
mwIndex *mxGetIr(const mxArray *a) { return a->ir; }
mwIndex *mxGetJc(const mxArray *a) { return a->jc; }
void mxSetNzmax(mxArray *a, mwSize n) { a->nzmax = n; }
void mxSetPr(mxArray *a, double *pr) { a->data = pr; }
void mxSetIr(mxArray *a, mwIndex *ir) { a->ir = ir; }

int mexPrintf(const char *fmt, ...) {
    va_list ap;
    va_start(ap, fmt);
    int n = vprintf(fmt, ap);
    va_end(ap);
    return n;
}

void mexErrMsgIdAndTxt(const char *id, const char *fmt, ...) {
    va_list ap;
    va_start(ap, fmt);
    fprintf(stderr, "error %s: ", id);
    vfprintf(stderr, fmt, ap);
    fprintf(stderr, "\n");
    va_end(ap);
    exit(1);
}

/* num2str: integers exactly; other values with 4 digits after the leading
 * one (MATLAB's default for scalars); vectors joined by two spaces. */
static void fmt_number(char *dst, size_t cap, double v) {
    if (v == (double)(long long)v && v < 1e15 && v > -1e15) {
        snprintf(dst, cap, "%lld", (long long)v);
    } else {
        snprintf(dst, cap, "%.5g", v);
    }
}

int mexCallMATLAB(int nlhs, mxArray *plhs[], int nrhs, mxArray *prhs[], const char *name) {
    (void)nrhs;
    if (strcmp(name, "num2str") == 0) {
        const mxArray *a = prhs[0];
        size_t n = a->dims[0] * a->dims[1];
        char buf[4096] = "";
        for (size_t i = 0; i < n; i++) {
            char one[64];
            double v = a->kind == K_INT32 ? (double)((int32_t *)a->data)[i]
                       : a->kind == K_LOGICAL ? (double)((mxLogical *)a->data)[i]
                                              : ((double *)a->data)[i];
            fmt_number(one, sizeof one, v);
            if (i) strcat(buf, "  ");
            strcat(buf, one);
        }
        plhs[0] = mxCreateString(buf);
        return 0;
    }
    if (strcmp(name, "waitbar") == 0 || strcmp(name, "close") == 0) {
        if (nlhs > 0) plhs[0] = mxCreateDoubleScalar(1.0);
        return 0;
    }
    fprintf(stderr, "harness: mexCallMATLAB(%s) not provided\n", name);
    return 1;
}

/* ---------------------------------------------------------------------- */
static void *read_file(const char *path, size_t *len) {
    FILE *f = fopen(path, "rb");
    if (!f) {
        fprintf(stderr, "harness: cannot open %s\n", path);
        exit(3);
    }
    fseek(f, 0, SEEK_END);
    long n = ftell(f);
    fseek(f, 0, SEEK_SET);
    char *buf = malloc((size_t)n + 1);
    if (fread(buf, 1, (size_t)n, f) != (size_t)n) {
        fprintf(stderr, "harness: short read %s\n", path);
        exit(3);
    }
    buf[n] = '\0';
    fclose(f);
    if (len) *len = (size_t)n;
    return buf;
}

static mxArray *new_struct(void) { return new_array(K_STRUCT); }
static void add_field(mxArray *s, const char *name, mxArray *v) {
    s->names = realloc(s->names, (s->nfields + 1) * sizeof(char *));
    s->fields = realloc(s->fields, (s->nfields + 1) * sizeof(mxArray *));
    s->names[s->nfields] = strdup(name);
    s->fields[s->nfields] = v;
    s->nfields++;
}

/* Reads whitespace-separated doubles. */
static double *parse_doubles(char **cur, size_t n) {
    double *v = malloc((n ? n : 1) * sizeof(double));
    for (size_t i = 0; i < n; i++) v[i] = strtod(*cur, cur);
    return v;
}

static char *next_line(char **cur) {
    char *s = *cur;
    if (!*s) return NULL;
    char *e = strchr(s, '\n');
    if (e) {
        *e = '\0';
        *cur = e + 1;
    } else {
        *cur = s + strlen(s);
    }
    return s;
}

int main(int argc, char **argv) {
    if (argc != 2) {
        fprintf(stderr, "usage: %s <dir>\n", argv[0]);
        return 2;
    }
    char path[4096];
    const char *dir = argv[1];

    /* mcGeo: dims, materials, bounds. */
    snprintf(path, sizeof path, "%s/geo.txt", dir);
    char *geo = read_file(path, NULL), *cur = geo;
    long nx = strtol(cur, &cur, 10), ny = strtol(cur, &cur, 10), nz = strtol(cur, &cur, 10);
    long nmat = strtol(cur, &cur, 10);
    next_line(&cur);
    mxArray *mcGeo = new_struct();
    mxArray *mat = new_array(K_CELL);
    mat->dims[0] = (mwSize)nmat;
    mat->dims[1] = 1;
    mat->data = blk_alloc((size_t)nmat * sizeof(mxArray *));
    for (long i = 0; i < nmat; i++) ((mxArray **)mat->data)[i] = mxCreateString(next_line(&cur));
    add_field(mcGeo, "material", mat);
    long nb[3] = {nx, ny, nz};
    const char *bn[3] = {"xBounds", "yBounds", "zBounds"};
    for (int k = 0; k < 3; k++) {
        double *b = parse_doubles(&cur, (size_t)nb[k] + 1);
        add_field(mcGeo, bn[k], new_doubles((size_t)nb[k] + 1, b));
        free(b);
    }
    free(geo);

    /* cubeRho, cubeMatIx. */
    size_t nvox = (size_t)nx * ny * nz, len;
    snprintf(path, sizeof path, "%s/rho.f64", dir);
    double *rho = read_file(path, &len);
    if (len != nvox * sizeof(double)) {
        fprintf(stderr, "harness: rho.f64 size\n");
        return 3;
    }
    mxArray *cubeRho = new_array(K_DOUBLE);
    cubeRho->ndim = 3;
    cubeRho->dims[0] = (mwSize)nx;
    cubeRho->dims[1] = (mwSize)ny;
    cubeRho->dims[2] = (mwSize)nz;
    cubeRho->data = blk_alloc(len);
    memcpy(cubeRho->data, rho, len);
    free(rho);
    snprintf(path, sizeof path, "%s/matix.i32", dir);
    int32_t *mix = read_file(path, &len);
    mxArray *cubeMatIx = new_array(K_INT32);
    cubeMatIx->ndim = 3;
    memcpy(cubeMatIx->dims, cubeRho->dims, sizeof cubeRho->dims);
    cubeMatIx->data = blk_alloc(len);
    memcpy(cubeMatIx->data, mix, len);
    free(mix);

    /* mcSrc. */
    snprintf(path, sizeof path, "%s/src.txt", dir);
    char *src = read_file(path, NULL);
    cur = src;
    long nbix = strtol(cur, &cur, 10), nbeams = strtol(cur, &cur, 10);
    mxArray *mcSrc = new_struct();
    add_field(mcSrc, "nBixels", mxCreateDoubleScalar((double)nbix));
    double *ib = parse_doubles(&cur, (size_t)nbix);
    add_field(mcSrc, "iBeam", new_doubles((size_t)nbix, ib));
    free(ib);
    const char *beam_fields[3] = {"xSource", "ySource", "zSource"};
    for (int k = 0; k < 3; k++) {
        double *v = parse_doubles(&cur, (size_t)nbeams);
        add_field(mcSrc, beam_fields[k], new_doubles((size_t)nbeams, v));
        free(v);
    }
    const char *bix_fields[9] = {"xCorner", "yCorner", "zCorner", "xSide1", "ySide1", "zSide1",
                                 "xSide2",  "ySide2",  "zSide2"};
    for (int k = 0; k < 9; k++) {
        double *v = parse_doubles(&cur, (size_t)nbix);
        add_field(mcSrc, bix_fields[k], new_doubles((size_t)nbix, v));
        free(v);
    }
    free(src);

    /* mcOpt: "name<TAB>d|s|b<TAB>value" lines. */
    snprintf(path, sizeof path, "%s/opt.txt", dir);
    char *opt = read_file(path, NULL);
    cur = opt;
    mxArray *mcOpt = new_struct();
    char *line;
    while ((line = next_line(&cur)) != NULL) {
        if (!*line) continue;
        char *name = strtok(line, "\t");
        char *type = strtok(NULL, "\t");
        char *val = strtok(NULL, "\t");
        if (!name || !type) continue;
        if (!val) val = "";
        if (type[0] == 's') {
            add_field(mcOpt, name, mxCreateString(val));
        } else if (type[0] == 'b') {
            mxArray *a = new_array(K_LOGICAL);
            a->data = blk_alloc(sizeof(mxLogical));
            ((mxLogical *)a->data)[0] = atoi(val) != 0;
            add_field(mcOpt, name, a);
        } else {
            double vals[16];
            size_t n = 0;
            char *c = val;
            while (n < 16) {
                char *e;
                double v = strtod(c, &e);
                if (e == c) break;
                vals[n++] = v;
                c = e;
            }
            add_field(mcOpt, name, new_doubles(n, vals));
        }
    }
    free(opt);

    const mxArray *prhs[5] = {cubeRho, cubeMatIx, mcGeo, mcSrc, mcOpt};
    mxArray *plhs[1] = {NULL};
    mexFunction(1, plhs, 5, prhs);

    mxArray *d = plhs[0];
    int64_t hdr[3] = {(int64_t)d->dims[0], (int64_t)d->dims[1], (int64_t)d->jc[d->dims[1]]};
    snprintf(path, sizeof path, "%s/dij.bin", dir);
    FILE *f = fopen(path, "wb");
    if (!f) return 3;
    fwrite(hdr, sizeof hdr, 1, f);
    for (mwSize j = 0; j <= d->dims[1]; j++) {
        int64_t v = (int64_t)d->jc[j];
        fwrite(&v, sizeof v, 1, f);
    }
    for (int64_t k = 0; k < hdr[2]; k++) {
        int64_t v = (int64_t)d->ir[k];
        fwrite(&v, sizeof v, 1, f);
    }
    fwrite(d->data, sizeof(double), (size_t)hdr[2], f);
    fclose(f);
    return 0;
}
