/*
 * Test oracle (test infrastructure only, see omc_oracle.h): FP64 CPU
 * restatement of the reference's omc_dosxyz transport.  Each function names
 * the reference routine it follows; arithmetic is written in the same
 * evaluation order and random numbers are drawn in the same sequence, so a
 * serial run reproduces the reference's serial build bit for bit.
 */
#include "omc_oracle.h"

#include <float.h>
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define RM 0.5109989461
#define MXGE OMC_MXGE
#define MXEKE OMC_MXEKE
#define MXSTACK 10000
#define SGMFP 1.0E-05
#define EPSEMFP 1.0E-5
#define SKIN_DEPTH_FOR_BCA 3
#define HC_INVERSE 80.65506856998
#define TWICE_HC2 0.000307444456
#define RAYCDFSIZE OMC_RAYCDFSIZE
#define MXE_SPIN OMC_MXE_SPIN
#define MXE_SPIN1 OMC_MXE_SPIN1
#define MXQ_SPIN OMC_MXQ_SPIN
#define MXU_SPIN OMC_MXU_SPIN
#define MXQ_MS OMC_MXQ_MS
#define MXU_MS OMC_MXU_MS
#define LAMBMAX_MS 1.0E5
#define QMIN_MS 1.0E-3
#define QMAX_MS 0.5
#ifndef M_PI
#define M_PI 3.14159265358979323846
#endif

/* ---------------------------------------------------------------------- */
/* RANMAR (omc_random.c:58-187).  Numbers come out one at a time; the
 * reference fills blocks of 128 but hands them out in the same order. */
typedef struct {
    int u[97];
    int i, j, c;
} ranmar_t;

static void ranmar_init(ranmar_t *r, int ixx, int jxx) {
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
        r->u[ii] = s;
    }
    r->c = 362436;
    r->i = 97;
    r->j = 33;
}

static inline int ranmar_int(ranmar_t *r) {
    int iopt = r->u[r->i - 1] - r->u[r->j - 1];
    if (iopt < 0) iopt += 16777216;
    r->u[r->i - 1] = iopt;
    r->i -= 1;
    r->j -= 1;
    if (r->i == 0) r->i = 97;
    else if (r->j == 0) r->j = 97;
    r->c -= 7654321;
    if (r->c < 0) r->c += 16777213;
    iopt -= r->c;
    if (iopt < 0) iopt += 16777216;
    return iopt;
}

void omc_oracle_ranmar(int ixx, int jxx, long long n, int *out) {
    ranmar_t r;
    ranmar_init(&r, ixx, jxx);
    for (long long i = 0; i < n; i++) out[i] = ranmar_int(&r);
}

/* ---------------------------------------------------------------------- */
typedef struct {
    const omc_tables *t;
    const omc_phantom *ph;
    const omc_regions *rg;
    const omc_source *src;
    int nsplit;
    double *endep; /* batch tally, shared between threads */
    const omc_beamlets *bl; /* beamlet source (omc_matrad), or NULL */
} ctx_t;

typedef struct {
    int np, npold;
    int iq[MXSTACK], ir[MXSTACK];
    double e[MXSTACK], x[MXSTACK], y[MXSTACK], z[MXSTACK];
    double u[MXSTACK], v[MXSTACK], w[MXSTACK], dnear[MXSTACK], wt[MXSTACK];
    ranmar_t rng;
    double ensrc;
    int overflow;
    const ctx_t *c;
} track_t;

typedef struct {
    double A, B, C, cosphi, sinphi;
} uphi_t;

typedef struct {
    int i, j;
} spinr_t;

typedef struct {
    int i, j;
    double omega2;
} mscats_t;

static inline double rnd(track_t *tk) { return ranmar_int(&tk->rng) * (1.0 / 16777216.0); }

/* ausgab (omc_dosxyz.c:683-694). */
static inline void ausgab(track_t *tk, double edep) {
    int np = tk->np;
    int irl = tk->ir[np];
    double endep = tk->wt[np] * edep;
    #pragma omp atomic
    tk->c->endep[irl] += endep;
}

/* howfar / hownear (omc_dosxyz.c:187-334). */
static void howfar(track_t *tk, int *idisc, int *irnew, double *ustep) {
    const omc_phantom *g = tk->c->ph;
    int np = tk->np;
    int irl = tk->ir[np];
    double dist;
    if (irl == 0) {
        *idisc = 1;
        return;
    }
    int ijmax = g->nx * g->ny, imax = g->nx;
    int irx = (irl - 1) % imax;
    int irz = (irl - 1 - irx) / ijmax;
    int iry = ((irl - 1 - irx) - irz * ijmax) / imax;
    if (tk->w[np] > 0.0) {
        dist = (g->zbounds[irz + 1] - tk->z[np]) / tk->w[np];
        if (dist < *ustep) {
            *ustep = dist;
            *irnew = (irz != g->nz - 1) ? irl + ijmax : 0;
        }
    } else if (tk->w[np] < 0.0) {
        dist = -(tk->z[np] - g->zbounds[irz]) / tk->w[np];
        if (dist < *ustep) {
            *ustep = dist;
            *irnew = (irz != 0) ? irl - ijmax : 0;
        }
    }
    if (tk->u[np] > 0.0) {
        dist = (g->xbounds[irx + 1] - tk->x[np]) / tk->u[np];
        if (dist < *ustep) {
            *ustep = dist;
            *irnew = (irx != g->nx - 1) ? irl + 1 : 0;
        }
    } else if (tk->u[np] < 0.0) {
        dist = -(tk->x[np] - g->xbounds[irx]) / tk->u[np];
        if (dist < *ustep) {
            *ustep = dist;
            *irnew = (irx != 0) ? irl - 1 : 0;
        }
    }
    if (tk->v[np] > 0.0) {
        dist = (g->ybounds[iry + 1] - tk->y[np]) / tk->v[np];
        if (dist < *ustep) {
            *ustep = dist;
            *irnew = (iry != g->ny - 1) ? irl + imax : 0;
        }
    } else if (tk->v[np] < 0.0) {
        dist = -(tk->y[np] - g->ybounds[iry]) / tk->v[np];
        if (dist < *ustep) {
            *ustep = dist;
            *irnew = (iry != 0) ? irl - imax : 0;
        }
    }
}

static double hownear(track_t *tk) {
    const omc_phantom *g = tk->c->ph;
    int np = tk->np;
    int irl = tk->ir[np];
    double tperp = 1.0E10;
    if (irl == 0) return 0.0;
    int ijmax = g->nx * g->ny, imax = g->nx;
    int irx = (irl - 1) % imax;
    int irz = (irl - 1 - irx) / ijmax;
    int iry = ((irl - 1 - irx) - irz * ijmax) / imax;
    tperp = fmin(tperp, g->xbounds[irx + 1] - tk->x[np]);
    tperp = fmin(tperp, tk->x[np] - g->xbounds[irx]);
    tperp = fmin(tperp, g->ybounds[iry + 1] - tk->y[np]);
    tperp = fmin(tperp, tk->y[np] - g->ybounds[iry]);
    tperp = fmin(tperp, g->zbounds[irz + 1] - tk->z[np]);
    tperp = fmin(tperp, tk->z[np] - g->zbounds[irz]);
    return tperp;
}

/* ---------------------------------------------------------------------- */
/* Stack helpers and rotations (ompmc.c:83-211). */
static void transfer(track_t *tk, int a, int b) {
    tk->x[a] = tk->x[b];
    tk->y[a] = tk->y[b];
    tk->z[a] = tk->z[b];
    tk->u[a] = tk->u[b];
    tk->v[a] = tk->v[b];
    tk->w[a] = tk->w[b];
    tk->ir[a] = tk->ir[b];
    tk->wt[a] = tk->wt[b];
    tk->dnear[a] = tk->dnear[b];
}

static void azimuth(track_t *tk, double *cphi, double *sphi) {
    double xphi, xphi2, yphi, yphi2, rhophi2;
    do {
        xphi = rnd(tk);
        xphi = 2.0 * xphi - 1.0;
        xphi2 = xphi * xphi;
        yphi = rnd(tk);
        yphi2 = yphi * yphi;
        rhophi2 = xphi2 + yphi2;
    } while (rhophi2 > 1.0);
    rhophi2 = 1 / rhophi2;
    *cphi = (xphi2 - yphi2) * rhophi2;
    *sphi = 2.0 * xphi * yphi * rhophi2;
}

static void rotate_new_dir(track_t *tk, int np, const uphi_t *up, double costhe, double sinthe) {
    double sinps2 = up->A * up->A + up->B * up->B;
    if (sinps2 < 1.0E-20) {
        tk->u[np] = sinthe * up->cosphi;
        tk->v[np] = sinthe * up->sinphi;
        tk->w[np] = up->C * costhe;
    } else {
        double sinpsi = sqrt(sinps2);
        double us = sinthe * up->cosphi;
        double vs = sinthe * up->sinphi;
        double sindel = up->B / sinpsi;
        double cosdel = up->A / sinpsi;
        tk->u[np] = up->C * cosdel * us - sindel * vs + up->A * costhe;
        tk->v[np] = up->C * sindel * us + cosdel * vs + up->B * costhe;
        tk->w[np] = -sinpsi * us + up->C * costhe;
    }
}

static void uphi21(track_t *tk, uphi_t *up, double costhe, double sinthe) {
    int np = tk->np;
    azimuth(tk, &up->cosphi, &up->sinphi);
    up->A = tk->u[np];
    up->B = tk->v[np];
    up->C = tk->w[np];
    rotate_new_dir(tk, np, up, costhe, sinthe);
}

static void uphi32(track_t *tk, uphi_t *up, double costhe, double sinthe) {
    int np = tk->np;
    transfer(tk, np, np - 1);
    rotate_new_dir(tk, np, up, costhe, sinthe);
}

static inline double pwlf(const double *c1, const double *c0, int idx, double lv) { return lv * c1[idx] + c0[idx]; }
static inline int pwlf_index(const double *c1, const double *c0, int idx, double lv) {
    return (int)(lv * c1[idx] + c0[idx]);
}

/* ---------------------------------------------------------------------- */
/* Photon interactions. */

/* rayleigh (ompmc.c:1102-1145).  The reference computes the CDF bin as
 * (int)rnno0 * dwi (always bin 0) and reads the tables of medium 0; both
 * are kept. */
static void rayleigh(track_t *tk, int imed, double eig, double gle, int lgle) {
    const omc_tables *t = tk->c->t;
    int ibin, ib;
    double xv, costhe, csqthe, sinthe, rnno0, rnno1;
    double pmax = pwlf(t->pmax1, t->pmax0, imed * MXGE + lgle, gle);
    double xmax = HC_INVERSE * eig;
    double dwi = (double)RAYCDFSIZE - 1.0;
    do {
        rnno1 = rnd(tk);
        do {
            rnno0 = rnd(tk);
            rnno0 *= pmax;
            ibin = (int)rnno0 * dwi;
            ib = t->i_array[ibin] - 1;
            if ((t->i_array[ibin + 1] - 1) > ib) {
                while (rnno0 >= t->fcum[ib + 1]) ib++;
            }
            rnno0 = (rnno0 - t->fcum[ib]) * t->c_array[ib];
            xv = t->xgrid[ib] * exp(log(1.0 + rnno0) * t->b_array[ib]);
        } while (xv >= xmax);
        xv /= eig;
        costhe = 1.0 - TWICE_HC2 * pow(xv, 2.0);
        csqthe = pow(costhe, 2.0);
    } while (2.0 * rnno1 >= (1.0 + csqthe));
    sinthe = sqrt(1.0 - csqthe);
    uphi_t up;
    uphi21(tk, &up, costhe, sinthe);
}

static double pair_rejection(const omc_tables *t, int imed, double xi, double esedei, double eseder, double tteig) {
    return 2.0 + 3.0 * (esedei + eseder) -
           4.0 * (esedei + eseder + 1.0 - 4.0 * pow((xi - 0.5), 2.0)) *
               (1.0 + 0.25 * log((pow(((1.0 + eseder) * (1.0 + esedei) / (2.0 * tteig)), 2.0)) +
                                 t->zbrang[imed] * pow(xi, 2.0)));
}

/* pair (ompmc.c:1429-1667). */
static void pair(track_t *tk, int imed) {
    const omc_tables *t = tk->c->t;
    int np = tk->np;
    double eig = tk->e[np];
    double ese1, ese2;
    int iq1, iq2, l, l1;
    tk->npold = np;
    if (eig <= 2.1) {
        double rnno0 = rnd(tk);
        double rnno1 = rnd(tk);
        ese2 = RM + 0.5 * rnno0 * (eig - 2.0 * RM);
        ese1 = eig - ese2;
        if (rnno1 < 0.5) {
            iq1 = -1;
            iq2 = 1;
        } else {
            iq1 = 1;
            iq2 = -1;
        }
    } else {
        double Amax, Bmax, delta, aux;
        if (eig < 50.0) {
            l = 4;
            l1 = l + 1;
            delta = 4.0 * t->delcm[imed] / eig;
            if (delta < 1.0) {
                Amax = t->dl1[imed * 8 + l] + delta * (t->dl2[imed * 8 + l] + delta * t->dl3[imed * 8 + l]);
                Bmax = t->dl1[imed * 8 + l1] + delta * (t->dl2[imed * 8 + l1] + delta * t->dl3[imed * 8 + l1]);
            } else {
                aux = log(delta + t->dl6[imed * 8 + l]);
                Amax = t->dl4[imed * 8 + l] + t->dl5[imed * 8 + l] * aux;
                Bmax = t->dl4[imed * 8 + l1] + t->dl5[imed * 8 + l1] * aux;
            }
            aux = 1.0 - 2.0 * RM / eig;
            aux = aux * aux;
            aux *= Amax / 3.0;
            aux /= (Bmax + aux);
        } else {
            l = 6;
            Amax = t->dl1[imed * 8 + l];
            Bmax = t->dl1[imed * 8 + l + 1];
            aux = t->bpar1[imed] * (1.0 - t->bpar0[imed] * RM / eig);
        }
        double eavail = eig - 2.0 * RM;
        double rejf, rejmax, rnno4;
        do {
            double br;
            double rnno0 = rnd(tk);
            double rnno1 = rnd(tk);
            rnno4 = rnd(tk);
            if (rnno0 > aux) {
                br = 0.5 * rnno1;
                rejmax = Bmax;
                l1 = l + 1;
            } else {
                double rnno2 = rnd(tk);
                double rnno3 = rnd(tk);
                br = 0.5 * (1.0 - fmax(fmax(rnno1, rnno2), rnno3));
                rejmax = Amax;
                l1 = l;
            }
            ese2 = br * eavail + RM;
            ese1 = eig - ese2;
            delta = (eig * t->delcm[imed]) / (ese2 * ese1);
            if (delta < 1.0)
                rejf = t->dl1[imed * 8 + l1] + delta * (t->dl2[imed * 8 + l1] + delta * t->dl3[imed * 8 + l1]);
            else
                rejf = t->dl4[imed * 8 + l1] + t->dl5[imed * 8 + l1] * log(delta + t->dl6[imed * 8 + l1]);
        } while (rnno4 * rejmax > rejf);
        ese1 = eig - ese2;
        rnno4 = rnd(tk);
        if (rnno4 < 0.5) {
            iq1 = -1;
            iq2 = 1;
        } else {
            iq1 = 1;
            iq2 = -1;
        }
    }
    tk->e[np] = ese1;
    tk->e[np + 1] = ese2;
    uphi_t up;
    for (int j = 0; j < 2; j++) {
        double ese = (j == 0) ? ese1 : ese2;
        double tteig = eig / RM;
        double ttese = ese / RM;
        double esedei = ttese / (tteig - ttese);
        double eseder = 1.0 / esedei;
        double ximin = 1.0 / (1.0 + pow((M_PI * ttese), 2.0));
        double rejmin = pair_rejection(t, imed, ximin, esedei, eseder, tteig);
        double ya = pow((2.0 / tteig), 2.0);
        double xitry = fmax(0.01, fmax(ximin, fmin(0.5, sqrt(ya / t->zbrang[imed]))));
        double galpha = 1.0 + 0.25 * log(ya + t->zbrang[imed] * xitry * xitry);
        double gbeta = 0.5 * t->zbrang[imed] * xitry / (ya + t->zbrang[imed] * xitry * xitry);
        galpha -= gbeta * (xitry - 0.5);
        double ximid = galpha / (3.0 * gbeta);
        if (galpha >= 0.0) ximid = 0.5 - ximid + sqrt(pow(ximid, 2.0) + 0.25);
        else ximid = 0.5 - ximid - sqrt(pow(ximid, 2.0) + 0.25);
        ximid = fmax(0.01, fmax(ximin, fmin(0.5, ximid)));
        double rejmid = pair_rejection(t, imed, ximid, esedei, eseder, tteig);
        double rejtop = 1.0 * fmax(rejmin, rejmid);
        double theta, rejtst, rejfactor, rtest;
        /* The reference rejects only when BOTH tests fail (ompmc.c:1641). */
        do {
            double xitst = rnd(tk);
            rejtst = pair_rejection(t, imed, xitst, esedei, eseder, tteig);
            rtest = rnd(tk);
            theta = sqrt(1.0 / xitst - 1.0) / ttese;
            rejfactor = rejtst / rejtop;
        } while ((rtest > rejfactor) && (theta >= M_PI));
        double sinthe = sin(theta);
        double costhe = cos(theta);
        if (j == 0) {
            uphi21(tk, &up, costhe, sinthe);
        } else {
            sinthe = -sinthe;
            np += 1;
            tk->np = np;
            uphi32(tk, &up, costhe, sinthe);
        }
    }
    tk->iq[np] = iq2;
    tk->iq[np - 1] = iq1;
}

/* compton (ompmc.c:1670-1783), free-electron Klein-Nishina. */
static void compton(track_t *tk) {
    int np = tk->np;
    double eig = tk->e[np];
    double ko = tk->e[np] / RM;
    double broi = 1.0 + 2.0 * ko;
    double bro = 1.0 / broi;
    int first_time = 1;
    double sinthe = 0.0, costhe = 0.0, br, rnno1, rnno2, rnno3, aux, rejf3, temp;
    double alph1 = 0.0, alph2 = 0.0, alpha = 0.0, rejmax = 0.0;
    tk->npold = np;
    do {
        if (ko > 2.0) {
            if (first_time) {
                alph1 = log(broi);
                alph2 = ko * (broi + 1.0) * pow(bro, 2.0);
                alpha = alph1 + alph2;
            }
            do {
                rnno1 = rnd(tk);
                rnno2 = rnd(tk);
                if (rnno1 * alpha < alph1) br = exp(alph1 * rnno2) * bro;
                else br = sqrt(rnno2 * pow(broi, 2.0) + (1.0 - rnno2)) * bro;
                temp = (1.0 - br) / (ko * br);
                sinthe = fmax(0.0, temp * (2.0 - temp));
                aux = 1.0 + pow(br, 2.0);
                rejf3 = aux - br * sinthe;
                rnno3 = rnd(tk);
            } while (rnno3 * aux > rejf3);
        } else {
            if (first_time) rejmax = broi + bro;
            do {
                rnno1 = rnd(tk);
                rnno2 = rnd(tk);
                br = bro + (1.0 - bro) * rnno1;
                temp = (1.0 - br) / (ko * br);
                sinthe = fmax(0.0, temp * (2.0 - temp));
                rejf3 = 1.0 + br * br - br * sinthe;
            } while (rnno2 * br * rejmax > rejf3);
        }
        first_time = 0;
    } while ((br < bro) || (br > 1));
    costhe = 1.0 - temp;
    sinthe = sqrt(sinthe);
    double esg = br * eig;
    double ese = eig - esg + RM;
    tk->e[np] = esg;
    uphi_t up;
    uphi21(tk, &up, costhe, sinthe);
    np += 1;
    tk->np = np;
    aux = 1.0 + br * br - 2.0 * br * costhe;
    if (aux > 1.0E-8) {
        costhe = (1.0 - br * costhe) / sqrt(aux);
        sinthe = (1.0 - costhe) * (1.0 + costhe);
        sinthe = (sinthe > 0.0) ? -sqrt(sinthe) : 0.0;
    } else {
        costhe = 0.0;
        sinthe = -1.0;
    }
    uphi32(tk, &up, costhe, sinthe);
    tk->e[np] = ese;
    tk->iq[np] = -1;
}

/* photo (ompmc.c:1786-1846): the photon becomes an electron of the full
 * photon energy (no binding); Sauter angular distribution. */
static void photo(track_t *tk) {
    const omc_regions *rg = tk->c->rg;
    int np = tk->np;
    tk->npold = np;
    tk->e[np] += RM;
    tk->iq[np] = -1;
    double eelec = tk->e[np];
    if (eelec > rg->ecut[tk->ir[np]]) {
        double beta = sqrt((eelec - RM) * (eelec + RM)) / eelec;
        double costhe, sinthe, sinth2, xi, rnpht2;
        double gamma = eelec / RM;
        double alpha = 0.5 * gamma - 0.5 + 1.0 / gamma;
        double ratio = beta / alpha;
        do {
            double rnpht = rnd(tk);
            rnpht = 2.0 * rnpht - 1.0;
            if (ratio <= 0.2) {
                double fkappa = rnpht + 0.5 * ratio * (1.0 - rnpht) * (1.0 + rnpht);
                if (gamma < 100.0) {
                    costhe = (beta + fkappa) / (1.0 + beta * fkappa);
                } else {
                    if (fkappa > 0.0)
                        costhe = 1.0 - (1.0 - fkappa) * (gamma - 3.0) / (2.0 * (1.0 + fkappa) * pow((gamma - 1.0), 3.0));
                    else
                        costhe = (beta + fkappa) / (1.0 + beta * fkappa);
                }
                xi = (1.0 + beta * fkappa) * pow(gamma, 2.0);
            } else {
                xi = pow(gamma, 2.0) * (1.0 + alpha * (sqrt(1.0 + ratio * (2.0 * rnpht + ratio)) - 1.0));
                costhe = (1.0 - 1.0 / xi) / beta;
            }
            sinth2 = fmax((1.0 - costhe) * (1.0 + costhe), 0.0);
            rnpht2 = rnd(tk);
        } while (rnpht2 > 0.5 * (1.0 + gamma) * sinth2 * xi / gamma);
        sinthe = sqrt(sinth2);
        uphi_t up;
        uphi21(tk, &up, costhe, sinthe);
    }
}

/* photon (ompmc.c:1849-2121), photon splitting included. */
static void photon(track_t *tk) {
    const omc_tables *t = tk->c->t;
    const omc_regions *rg = tk->c->rg;
    int np = tk->np;
    int irl = tk->ir[np];
    int irold, irnew, idisc;
    int imed = rg->med[irl];
    double rhof, tstep, ustep, edep;
    double eig = tk->e[np];
    double dpmfp, dpmfp_old, gmfpr0 = 0.0, gmfp = 0.0, gbr1, gbr2, rnno;
    int nsplit = tk->c->nsplit, i_survive_s, ip;
    double d_eta, eta_prime, a_survive;
    double xsave, ysave, zsave, usave, vsave, wsave, esave, wtsave;
    int irsave;

    if (eig <= rg->pcut[irl] || tk->wt[np] == 0) {
        edep = eig;
        ausgab(tk, edep);
        tk->np -= 1;
        return;
    }
    int lgle = 0;
    double gle = log(eig);
    double cohfac = 0.0;
    int ptrans;

start_mfp_loop:
    rnno = rnd(tk);
    rnno /= (double)nsplit;
    d_eta = 1.0 / (double)nsplit;
    eta_prime = 1.0 - rnno + d_eta;
    xsave = tk->x[np];
    ysave = tk->y[np];
    zsave = tk->z[np];
    usave = tk->u[np];
    vsave = tk->v[np];
    wsave = tk->w[np];
    esave = tk->e[np];
    wtsave = tk->wt[np] / (double)nsplit;
    irsave = tk->ir[np];
    np -= 1;
    rnno = rnd(tk);
    a_survive = rnno * nsplit;
    i_survive_s = (int)a_survive;
    dpmfp_old = 0.0;
    for (int isplit = 0; isplit < nsplit; isplit++) {
        ptrans = 1;
        eta_prime -= d_eta;
        if (eta_prime <= 0.0) goto end_mfp_loop;
        dpmfp = -log(eta_prime) - dpmfp_old;
        dpmfp_old += dpmfp;
        np += 1;
        tk->np = np;
        if (np >= MXSTACK) {
            tk->overflow = 1;
            tk->np = -1;
            return;
        }
        tk->x[np] = xsave;
        tk->y[np] = ysave;
        tk->z[np] = zsave;
        tk->u[np] = usave;
        tk->v[np] = vsave;
        tk->w[np] = wsave;
        tk->e[np] = esave;
        tk->wt[np] = wtsave;
        tk->ir[np] = irsave;
        tk->iq[np] = 0;
        irl = tk->ir[np];
        irold = irl;
        imed = rg->med[irl];
        do {
            if (imed != -1) {
                lgle = pwlf_index(t->ge1, t->ge0, imed, gle) - 1;
                gmfpr0 = pwlf(t->gmfp1, t->gmfp0, imed * MXGE + lgle, gle);
                rhof = rg->rhof[irl];
                gmfp = gmfpr0 / rhof;
                cohfac = pwlf(t->cohe1, t->cohe0, imed * MXGE + lgle, gle);
                gmfp *= cohfac;
                tstep = gmfp * dpmfp;
            } else {
                tstep = 1.0E8;
            }
            irnew = irl;
            idisc = 0;
            ustep = tstep;
            howfar(tk, &idisc, &irnew, &ustep);
            edep = 0.0;
            tk->x[np] += ustep * tk->u[np];
            tk->y[np] += ustep * tk->v[np];
            tk->z[np] += ustep * tk->w[np];
            if (idisc > 0) {
                np -= 1;
                tk->np = np;
                if (np < 0) return;
                goto end_mfp_loop;
            }
            if (imed != -1) dpmfp = fmax(0.0, dpmfp - ustep / gmfp);
            if (irnew != irold) {
                tk->ir[np] = irnew;
                irl = irnew;
                irold = irnew;
                imed = rg->med[irl];
            }
            if (imed != -1 && dpmfp <= SGMFP) ptrans = 0;
        } while (ptrans);
        xsave = tk->x[np];
        ysave = tk->y[np];
        zsave = tk->z[np];
        irsave = tk->ir[np];
        rnno = rnd(tk);
        if (rnno <= 1.0 - cohfac) {
            if (isplit != i_survive_s) {
                np -= 1;
                tk->np = np;
                continue;
            } else {
                tk->wt[np] *= nsplit;
                rayleigh(tk, imed, eig, gle, lgle);
                continue;
            }
        } else {
            rnno = rnd(tk);
            gbr1 = pwlf(t->gbr11, t->gbr10, imed * MXGE + lgle, gle);
            if (rnno <= gbr1 && eig > 2.0 * RM) {
                pair(tk, imed);
                np = tk->np;
            } else {
                gbr2 = pwlf(t->gbr21, t->gbr20, imed * MXGE + lgle, gle);
                if (rnno < gbr2) {
                    compton(tk);
                    np = tk->np;
                } else {
                    photo(tk);
                    np = tk->np;
                }
            }
        }
        /* Scattered photons of non-surviving splits are killed; the
         * survivor takes the weight of the original photon. */
        ip = tk->npold;
        do {
            if (tk->iq[ip] == 0) {
                if (isplit != i_survive_s) {
                    if (ip < np) {
                        tk->e[ip] = tk->e[np];
                        tk->iq[ip] = tk->iq[np];
                        tk->u[ip] = tk->u[np];
                        tk->v[ip] = tk->v[np];
                        tk->w[ip] = tk->w[np];
                        tk->wt[ip] = tk->wt[np];
                    }
                    np -= 1;
                } else {
                    tk->wt[ip] *= nsplit;
                    ip += 1;
                }
            } else {
                ip += 1;
            }
        } while (ip <= np);
        tk->np = np;
    }
end_mfp_loop:
    if (np < 0) return;
    if (tk->iq[np] == 0) {
        eig = tk->e[np];
        irl = tk->ir[np];
        imed = rg->med[irl];
        if (eig <= rg->pcut[irl]) {
            edep = eig;
            ausgab(tk, edep);
            np -= 1;
            tk->np = np;
            return;
        }
        gle = log(eig);
        goto start_mfp_loop;
    }
}

/* ---------------------------------------------------------------------- */
/* Electron physics. */

/* spinRejection (ompmc.c:3097-3168). */
static double spin_rejection(track_t *tk, int imed, int qel, double elke, double beta2, double q1, double cost,
                             int *spin_index, int is_single, spinr_t *sr) {
    const omc_tables *t = tk->c->t;
    int k;
    double ai, aj, ak, qq1, xi, rnno;
    if (*spin_index) {
        *spin_index = 0;
        if (beta2 >= t->b2spin_min) {
            ai = (beta2 - t->b2spin_min) * t->dbeta2i;
            sr->i = (int)ai;
            ai -= (double)sr->i;
            sr->i += MXE_SPIN + 1;
        } else if (elke > t->espml) {
            ai = (elke - t->espml) * t->dleneri;
            sr->i = (int)ai;
            ai -= sr->i;
        } else {
            sr->i = 0;
            ai = -1.0f;
        }
        rnno = rnd(tk);
        if (rnno < ai) sr->i += 1;
        if (is_single) {
            sr->j = 0;
        } else {
            qq1 = 2.0 * q1;
            qq1 = qq1 / (1.0 + qq1);
            aj = qq1 * t->dqq1i;
            sr->j = (int)aj;
            if (sr->j >= MXQ_SPIN) {
                sr->j = MXQ_SPIN;
            } else {
                aj -= (double)sr->j;
                rnno = rnd(tk);
                if (rnno < aj) sr->j += 1;
            }
        }
    }
    xi = sqrt(0.5 * (1.0 - cost));
    ak = xi * MXU_SPIN;
    k = (int)ak;
    ak -= (double)k;
    size_t base = (size_t)imed * 2 * (MXE_SPIN1 + 1) * (MXQ_SPIN + 1) * (MXU_SPIN + 1) +
                  (size_t)qel * (MXE_SPIN1 + 1) * (MXQ_SPIN + 1) * (MXU_SPIN + 1) +
                  (size_t)sr->i * (MXQ_SPIN + 1) * (MXU_SPIN + 1) + (size_t)sr->j * (MXU_SPIN + 1);
    double r1 = t->spin_rej[base + k];
    double r2 = t->spin_rej[base + k + 1];
    return (1.0 - ak) * (r1) + ak * r2;
}

/* sscat (ompmc.c:3170-3199). */
static void sscat(track_t *tk, int imed, int qel, double chia2, double elke, double beta2, double *cost,
                  double *sint) {
    int spin_index = 1;
    spinr_t sr;
    double xi, rejf, rnno;
    do {
        xi = rnd(tk);
        xi = 2.0 * chia2 * xi / (1.0 - xi + chia2);
        *cost = 1.0 - xi;
        rejf = spin_rejection(tk, imed, qel, elke, beta2, 0, *cost, &spin_index, 1, &sr);
        rnno = rnd(tk);
    } while (rnno > rejf);
    *sint = sqrt(xi * (2.0 - xi));
}

/* mscat (ompmc.c:3606-3785).  The reference's q-surface interpolation uses
 * du = ums[k] - ums[k] = 0 (so u = ums[k]); the draw is kept.  For
 * lambda > LAMBMAX_MS the reference leaves the angle unset; here cost = 1. */
static void mscat(track_t *tk, int imed, int qel, int *spin_index, int *find_index, double elke, double beta2,
                  double q1, double lambda, double chia2, double *cost, double *sint, mscats_t *ms, spinr_t *sr) {
    const omc_tables *t = tk->c->t;
    double xi, rejf, rnno;
    double explambda = exp(-lambda);
    if (lambda <= 13.8) {
        double sprob = rnd(tk);
        if (sprob < explambda) {
            *cost = 1.0;
            *sint = 0.0;
            return;
        }
        double wsum = (1.0 + lambda) * explambda;
        if (sprob < wsum) {
            do {
                xi = rnd(tk);
                xi = 2.0 * chia2 * xi / (1.0 - xi + chia2);
                *cost = 1.0 - xi;
                rejf = spin_rejection(tk, imed, qel, elke, beta2, q1, *cost, spin_index, 0, sr);
                rnno = rnd(tk);
            } while (rnno > rejf);
            *sint = sqrt(xi * (2.0 - xi));
            return;
        }
        if (lambda <= 1) {
            int icount = 0;
            double wprob = explambda, sinz, cosz, phi;
            wsum = explambda;
            *cost = 1.0;
            *sint = 0.0;
            do {
                icount += 1;
                if (icount > 20) break;
                wprob = wprob * lambda / icount;
                wsum = wsum + wprob;
                do {
                    xi = rnd(tk);
                    xi = 2.0 * chia2 * xi / (1.0 - xi + chia2);
                    cosz = 1.0 - xi;
                    rejf = spin_rejection(tk, imed, qel, elke, beta2, q1, cosz, spin_index, 0, sr);
                    rnno = rnd(tk);
                } while (rnno > rejf);
                sinz = xi * (2.0 - xi);
                if (sinz > 1.0E-20) {
                    sinz = sqrt(sinz);
                    xi = rnd(tk);
                    phi = xi * 6.2831853;
                    *cost = (*cost) * cosz - *sint * sinz * cos(phi);
                    *sint = sqrt(fmax(0.0, (double)((1.0 - (*cost)) * (1.0 + (*cost)))));
                }
            } while (wsum <= sprob);
            return;
        }
    }
    if (lambda <= LAMBMAX_MS) {
        double ai, aj;
        double llmbda = log(lambda);
        if (*find_index) {
            ai = llmbda * t->dllambi;
            ms->i = (int)ai;
            ai -= (double)ms->i;
            xi = rnd(tk);
            if (xi < ai) ms->i += 1;
            if (q1 < QMIN_MS) {
                ms->j = 0;
            } else if (q1 < QMAX_MS) {
                aj = q1 * t->dqmsi;
                ms->j = (int)aj;
                aj -= (double)ms->j;
                xi = rnd(tk);
                if (xi < aj) ms->j += 1;
            } else {
                ms->j = MXQ_MS;
            }
            if (llmbda < 2.2299)
                ms->omega2 = chia2 * (lambda + 4.0) *
                             (1.347006 + llmbda * (0.209364 - llmbda * (0.45525 - llmbda * (0.50142 - 0.081234 * llmbda))));
            else
                ms->omega2 = chia2 * (lambda + 4.0) *
                             (-2.77164 + llmbda * (2.94874 - llmbda * (0.1535754 - llmbda * 0.00552888)));
            *find_index = 0;
        }
        int k;
        double a, ak, u, du, x1;
        size_t row = (size_t)ms->i * (MXQ_MS + 1) * (MXU_MS + 1) + (size_t)ms->j * (MXU_MS + 1);
        do {
            xi = rnd(tk);
            ak = xi * MXU_MS;
            k = ak;
            ak -= k;
            if (ak > t->wms[row + k]) k = t->ims[row + k];
            a = t->fms[row + k];
            u = t->ums[row + k];
            du = t->ums[row + k] - u;
            xi = rnd(tk);
            if (fabs(a) < 0.2) {
                x1 = 0.5 * (1.0 - xi) * a;
                u += xi * du * (1.0 + x1 * (1.0 - xi * a));
            } else {
                u -= du / a * (1.0 - sqrt(1.0 + xi * a * (2.0 + a)));
            }
            xi = ms->omega2 * u / (1.0 + 0.5 * ms->omega2 - u);
            if (xi > 1.99999) xi = 1.99999;
            *cost = 1.0 - xi;
            rejf = spin_rejection(tk, imed, qel, elke, beta2, q1, *cost, spin_index, 0, sr);
            rnno = rnd(tk);
        } while (rnno > rejf);
        *sint = sqrt(xi * (2.0 - xi));
    } else {
        *cost = 1.0;
        *sint = 0.0;
    }
}

/* msdist (ompmc.c:3787-3976): PRESTA-II substep angles and lateral
 * displacement. */
static double msdist(track_t *tk, int imed, int iq, double rhof, double de, double tustep, double eke, double *x_final,
                     double *y_final, double *z_final, double *u_final, double *v_final, double *w_final) {
    const omc_tables *t = tk->c->t;
    int qel = (1 + iq) / 2;
    mscats_t ms;
    spinr_t sr;
    double blccc = t->blcc[imed];
    double xcccc = t->xcc[imed];
    double e = eke - 0.5 * de;
    double tau = e / RM;
    double tau2 = pow(tau, 2.0);
    double epsilon = de / eke;
    double epsilonp = de / e;
    e *= (1.0 - pow(epsilonp, 2.0) * (6.0 + 10.0 * tau + 5.0 * tau2) / (24.0 * tau2 + 72.0 * tau + 48.0));
    double p2 = e * (e + 2.0 * RM);
    double beta2 = p2 / (p2 + pow(RM, 2.0));
    double chia2 = xcccc / (4.0 * p2 * blccc);
    double lambda = 0.5 * tustep * rhof * blccc / beta2;
    double temp2 = 0.166666 * (4.0 + tau * (6.0 + tau * (7.0 + tau * (4.0 + tau)))) *
                   (epsilonp / ((tau + 1.0) * (tau + 2.0))) * (epsilonp / ((tau + 1.0) * (tau + 2.0)));
    lambda *= (1.0 - temp2);
    double elke = log(e);
    int lelke = pwlf_index(t->eke1, t->eke0, imed, elke) - 1;
    if (lelke < 0) {
        lelke = 0;
        elke = (1.0 - t->eke0[imed]) / t->eke1[imed];
    }
    int ix = MXEKE * imed + lelke;
    double etap, xi_corr, gamma;
    if (qel == 0) {
        etap = pwlf(t->etae_ms1, t->etae_ms0, ix, elke);
        xi_corr = pwlf(t->q1ce_ms1, t->q1ce_ms0, ix, elke);
        gamma = pwlf(t->q2ce_ms1, t->q2ce_ms0, ix, elke);
    } else {
        etap = pwlf(t->etap_ms1, t->etap_ms0, ix, elke);
        xi_corr = pwlf(t->q1cp_ms1, t->q1cp_ms0, ix, elke);
        gamma = pwlf(t->q2cp_ms1, t->q2cp_ms0, ix, elke);
    }
    double ms_corr = pwlf(t->blcce1, t->blcce0, ix, elke);
    chia2 *= etap;
    lambda /= (etap * (1.0 + chia2));
    lambda *= ms_corr;
    double chilog = log(1.0 + 1.0 / chia2);
    double q1 = 2.0 * chia2 * (chilog * (1.0 + chia2) - 1.0);
    gamma = 6.0 * chia2 * (1.0 + chia2) * (chilog * (1.0 + 2.0 * chia2) - 2.0) / q1 * gamma;
    double xi = q1 * lambda;
    int find_index = 1, spin_index = 1;
    double w1, sint1, cphi1, sphi1, w2, sint2, cphi2, sphi2;
    mscat(tk, imed, qel, &spin_index, &find_index, elke, beta2, xi, lambda, chia2, &w1, &sint1, &ms, &sr);
    azimuth(tk, &cphi1, &sphi1);
    mscat(tk, imed, qel, &spin_index, &find_index, elke, beta2, xi, lambda, chia2, &w2, &sint2, &ms, &sr);
    azimuth(tk, &cphi2, &sphi2);
    double u2 = sint2 * cphi2;
    double v2 = sint2 * sphi2;
    double u2p = w1 * u2 + sint1 * w2;
    double us = u2p * cphi1 - v2 * sphi1;
    double vs = u2p * sphi1 + v2 * cphi1;
    double ws = w1 * w2 - sint1 * u2;
    xi *= 2 * xi_corr;
    double eta = rnd(tk);
    double eta1 = 0.5 * (1.0 - eta);
    double delta = 0.9082483 - (0.1020621 - 0.0263747 * gamma) * xi;
    double temp1 = 2.0 + tau;
    double temp = (2.0 + tau * temp1) / ((tau + 1.0) * temp1);
    temp -= (tau + 1.0) / ((tau + 2.0) * (chilog * (1.0 + chia2) - 1.0));
    temp *= epsilonp;
    temp1 = 1.0 - temp;
    delta += 0.40824829 * (epsilon * (tau + 1.0) /
                               ((tau + 2.0) * (chilog * (1.0 + chia2) - 1.0) * (chilog * (1.0 + 2.0 * chia2) - 2.0)) -
                           0.25 * pow(temp, 2.0));
    double b = eta * delta;
    double c = eta * (1.0 - delta);
    double w1v2 = w1 * v2;
    double ut = b * sint1 * cphi1 + c * (cphi1 * u2 - sphi1 * w1v2) + eta1 * us * temp1;
    double vt = b * sint1 * sphi1 + c * (sphi1 * u2 + cphi1 * w1v2) + eta1 * vs * temp1;
    double wt = eta1 * (1.0 + temp) + b * w1 + c * w2 + eta1 * ws * temp1;
    double ustep = tustep * sqrt(ut * ut + vt * vt + wt * wt);
    int np = tk->np;
    double x0 = tk->x[np], y0 = tk->y[np], z0 = tk->z[np];
    double u0 = tk->u[np], v0 = tk->v[np], w0 = tk->w[np];
    double sint02 = u0 * u0 + v0 * v0;
    if (sint02 > 1.0E-20) {
        double sint0 = sqrt(sint02);
        double sint0i = 1.0 / sint0;
        double cphi0 = sint0i * u0;
        double sphi0 = sint0i * v0;
        u2p = w0 * us + sint0 * ws;
        ws = w0 * ws - sint0 * us;
        us = u2p * cphi0 - vs * sphi0;
        vs = u2p * sphi0 + vs * cphi0;
        u2p = w0 * ut + sint0 * wt;
        wt = w0 * wt - sint0 * ut;
        ut = u2p * cphi0 - vt * sphi0;
        vt = u2p * sphi0 + vt * cphi0;
    } else {
        wt = w0 * wt;
        ws = w0 * ws;
    }
    *x_final = x0 + tustep * ut;
    *y_final = y0 + tustep * vt;
    *z_final = z0 + tustep * wt;
    *u_final = us;
    *v_final = vs;
    *w_final = ws;
    return ustep;
}

/* computeDrange / computeEloss (ompmc.c:3979-4108). */
static double drange(const omc_tables *t, int imed, int iq, int lelke, double ekei, double ekef, double elkei,
                     double elkef) {
    double dedxmid, aux;
    double fedep = 1.0 - ekef / ekei;
    double elktmp = 0.5 * (elkei + elkef + 0.25 * fedep * fedep * (1.0 + fedep * (1.0 + 0.875 * fedep)));
    int ix = MXEKE * imed + lelke;
    if (iq < 0) {
        dedxmid = pwlf(t->ededx1, t->ededx0, ix, elktmp);
        dedxmid = 1.0 / dedxmid;
        aux = t->ededx1[ix] * dedxmid;
    } else {
        dedxmid = pwlf(t->pdedx1, t->pdedx0, ix, elktmp);
        dedxmid = 1.0 / dedxmid;
        aux = t->pdedx1[ix] * dedxmid;
    }
    aux = aux * (1.0 + 2.0 * aux) * fedep * fedep / (6.0 * (2.0 - fedep) * (2.0 - fedep));
    return fedep * ekei * dedxmid * (1.0 + aux);
}

static double eloss(const omc_tables *t, int imed, int iq, double rhof, double tustep, double range, double eke,
                    double elke, int lelke) {
    double aux, dedxmid, de, fedep, elktmp, eketmp;
    int lelktmp;
    int qel = (1 + iq) / 2;
    const double *rng_ep = t->range_ep + (size_t)qel * t->nmed * MXEKE + (size_t)imed * MXEKE;
    double tuss = range - rng_ep[lelke] / rhof;
    if (tuss >= tustep) {
        int ix = imed * MXEKE + lelke;
        if (iq < 0) {
            dedxmid = pwlf(t->ededx1, t->ededx0, ix, elke);
            aux = t->ededx1[ix] / dedxmid;
        } else {
            dedxmid = pwlf(t->pdedx1, t->pdedx0, ix, elke);
            aux = t->pdedx1[ix] / dedxmid;
        }
        de = dedxmid * tustep * rhof;
        fedep = de / eke;
        de *= (1.0 - 0.5 * fedep * aux * (1.0 - 0.333333 * fedep * (aux - 1.0 - 0.25 * fedep * (2.0 - aux * (4.0 - aux)))));
    } else {
        lelktmp = lelke;
        tuss = (range - tustep) * rhof;
        if (tuss <= 0) {
            de = eke - t->te[imed] * 0.99;
        } else {
            while (tuss < rng_ep[lelktmp]) lelktmp -= 1;
            elktmp = (lelktmp + 2 - t->eke0[imed]) / t->eke1[imed];
            eketmp = t->e_array[imed * MXEKE + lelktmp + 1];
            tuss = (rng_ep[lelktmp + 1] - tuss) / rhof;
            int ix = MXEKE * imed + lelktmp;
            if (iq < 0) {
                dedxmid = pwlf(t->ededx1, t->ededx0, ix, elktmp);
                aux = t->ededx1[ix] / dedxmid;
            } else {
                dedxmid = pwlf(t->pdedx1, t->pdedx0, ix, elktmp);
                aux = t->pdedx1[ix] / dedxmid;
            }
            de = dedxmid * tuss * rhof;
            fedep = de / eketmp;
            de *= (1.0 - 0.5 * fedep * aux * (1.0 - 0.333333 * fedep * (aux - 1.0 - 0.25 * fedep * (2.0 - aux * (4.0 - aux)))));
            de += eke - eketmp;
        }
    }
    return de;
}

/* Photons created by brems/annih/rannih are Russian-rouletted when
 * splitting is on (ompmc.c:4151-4164, 4340-4353, 4629-4642). */
static void roulette_photons(track_t *tk, int draw_for_all) {
    int nsplit = tk->c->nsplit;
    (void)draw_for_all;
    if (nsplit > 1) {
        for (int ip = tk->npold; ip <= tk->np; ip++) {
            if (tk->iq[ip] == 0) {
                double r = rnd(tk);
                if (r * (double)nsplit > 1.0) {
                    tk->wt[ip] = 0.0;
                    tk->e[ip] = 0.0;
                } else {
                    tk->wt[ip] *= nsplit;
                }
            }
        }
    }
}

/* rannih (ompmc.c:4111-4167): two back-to-back 511 keV photons.  The
 * reference draws one number it does not use before the azimuth. */
static void rannih(track_t *tk) {
    double rnno;
    int np = tk->np;
    tk->npold = np;
    rnno = rnd(tk);
    double costhe = 2.0 * rnno - 1;
    double sinthe = sqrt(fmax(0.0, (1.0 - costhe) * (1.0 + costhe)));
    rnno = rnd(tk);
    (void)rnno;
    double cosphi, sinphi;
    azimuth(tk, &cosphi, &sinphi);
    tk->e[np] = RM;
    tk->iq[np] = 0;
    tk->u[np] = sinthe * cosphi;
    tk->v[np] = sinthe * sinphi;
    tk->w[np] = costhe;
    np += 1;
    tk->e[np] = RM;
    tk->iq[np] = 0;
    transfer(tk, np, np - 1);
    tk->u[np] = -1.0 * tk->u[np - 1];
    tk->v[np] = -1.0 * tk->v[np - 1];
    tk->w[np] = -1.0 * tk->w[np - 1];
    tk->np = np;
    roulette_photons(tk, 1);
}

/* brems (ompmc.c:4170-4356): Bethe-Heitler (Coulomb corrected above 50 MeV)
 * energy, 2BS-style angle. */
static void brems(track_t *tk) {
    const omc_tables *t = tk->c->t;
    const omc_regions *rg = tk->c->rg;
    int np = tk->np;
    int irl = tk->ir[np];
    int imed = rg->med[irl];
    double eie = tk->e[np];
    double phi1, phi2;
    tk->npold = np;
    int l = (eie < 50.0) ? 1 : 3;
    int l1 = l + 1;
    double ekin = eie - RM;
    double brmin = t->ap[imed] / ekin;
    double waux = -log(brmin);
    double a, b, c, sinpsi, sindel = 0.0, cosdel = 0.0, ztarg, tteie, y2maxi, z2maxi;
    a = tk->u[np];
    b = tk->v[np];
    c = tk->w[np];
    sinpsi = a * a + b * b;
    if (sinpsi > 1.0E-20) {
        sinpsi = sqrt(sinpsi);
        sindel = b / sinpsi;
        cosdel = a / sinpsi;
    }
    ztarg = t->zbrang[imed];
    tteie = eie / RM;
    double beta = sqrt((tteie - 1.0) * (tteie + 1.0)) / tteie;
    double y2max = 2.0 * beta * (1.0 + beta) * tteie * tteie;
    y2maxi = 1.0 / y2max;
    double z2max = y2max + 1.0;
    z2maxi = sqrt(z2max);
    double aux, br, delta, rnno06, rnno07, rejf, ese, esg;
    do {
        rnno06 = rnd(tk);
        rnno07 = rnd(tk);
        br = brmin * exp(rnno06 * waux);
        esg = ekin * br;
        ese = eie - esg;
        delta = esg / eie / ese * t->delcm[imed];
        aux = ese / eie;
        if (delta < 1.0) {
            phi1 = t->dl1[imed * 8 + l - 1] + delta * (t->dl2[imed * 8 + l - 1] + delta * t->dl3[imed * 8 + l - 1]);
            phi2 = t->dl1[imed * 8 + l1 - 1] + delta * (t->dl2[imed * 8 + l1 - 1] + delta * t->dl3[imed * 8 + l1 - 1]);
        } else {
            phi1 = t->dl4[imed * 8 + l - 1] + t->dl5[imed * 8 + l - 1] * log(delta + t->dl6[imed * 8 + l - 1]);
            phi2 = phi1;
        }
        rejf = (1.0 + pow(aux, 2.0)) * phi1 - 2.0 * aux * phi2 / 3.0;
    } while (rnno07 >= rejf);
    np += 1;
    tk->e[np] = esg;
    tk->iq[np] = 0;
    transfer(tk, np, np - 1);
    double y2tst, ttese = ese / RM, esedei = ttese / tteie, rejmax;
    double rjarg1 = 1.0 + esedei * esedei;
    double rjarg2 = rjarg1 + 2.0 * esedei;
    double rjarg3;
    double rtest = 1.0, rejtst = 0.0;
    aux = 2.0 * ese * tteie / esg;
    aux = aux * aux;
    double aux1 = aux * ztarg;
    if (aux1 > 10.0) rjarg3 = -log(t->zbrang[imed]) + (1.0 - aux1) / pow(aux1, 2.0);
    else rjarg3 = log(aux / (1.0 + aux1));
    rejmax = rjarg1 * rjarg3 - rjarg2;
    while (rtest >= rejtst) {
        y2tst = rnd(tk);
        rtest = rnd(tk);
        double aux3 = z2maxi / (y2tst + (1.0 - y2tst) * z2maxi);
        rtest = rtest * aux3 * rejmax;
        y2tst = pow(aux3, 2.0) - 1.0;
        double y2tst1 = esedei * y2tst / pow(aux3, 4.0);
        double aux4 = 16.0 * y2tst1 - rjarg2;
        double aux5 = rjarg1 - 4.0 * y2tst1;
        if (rtest < aux4 + aux5 * rjarg3) break;
        double aux2 = log(aux / (1.0 + aux1 / pow(aux3, 4.0)));
        rejtst = aux4 + aux5 * aux2;
    }
    double costhe = 1.0 - 2.0 * y2tst * y2maxi;
    double sinthe = sqrt(fmax(0.0, (1.0 - pow(costhe, 2.0))));
    double cphi, sphi;
    azimuth(tk, &cphi, &sphi);
    if (sinpsi >= 1.0E-10) {
        double us = sinthe * cphi;
        double vs = sinthe * sphi;
        tk->u[np] = c * cosdel * us - sindel * vs + a * costhe;
        tk->v[np] = c * sindel * us + cosdel * vs + b * costhe;
        tk->w[np] = c * costhe - sinpsi * us;
    } else {
        tk->u[np] = sinthe * cphi;
        tk->v[np] = sinthe * sphi;
        tk->w[np] = c * costhe;
    }
    tk->e[np - 1] = ese;
    tk->np = np;
    roulette_photons(tk, 0);
}

/* moller (ompmc.c:4359-4435). */
static void moller(track_t *tk) {
    const omc_tables *t = tk->c->t;
    const omc_regions *rg = tk->c->rg;
    int np = tk->np;
    int irl = tk->ir[np];
    int imed = rg->med[irl];
    double eie = tk->e[np];
    double ekin = eie - RM;
    tk->npold = np;
    if (ekin <= 2.0 * t->te[imed]) return;
    double t0 = ekin / RM;
    double e0 = t0 + 1.0;
    double extrae = eie - t->thmoll[imed];
    double g2 = pow(t0, 2.0) / pow(e0, 2.0);
    double g3 = (2.0 * t0 + 1.0) / pow(e0, 2.0);
    double br, gmax = (1.0 + 1.25 * g2), rejf4, r, rnno27, rnno28;
    do {
        rnno27 = rnd(tk);
        br = t->te[imed] / (ekin - extrae * rnno27);
        r = br / (1.0 - br);
        rnno28 = rnd(tk);
        rejf4 = (1.0 + g2 * pow(br, 2.0) + r * (r - g3));
        rnno28 *= gmax;
    } while (rnno28 > rejf4);
    double ekse2 = br * ekin;
    double ese1 = eie - ekse2;
    double ese2 = ekse2 + RM;
    tk->e[np] = ese1;
    tk->e[np + 1] = ese2;
    double h1 = (eie + RM) / ekin;
    double costh = h1 * (ese1 - RM) / (ese1 + RM);
    double sinthe = sqrt(1.0 - costh);
    double costhe = sqrt(costh);
    uphi_t up;
    uphi21(tk, &up, costhe, sinthe);
    np += 1;
    tk->np = np;
    tk->iq[np] = -1;
    costh = h1 * (ese2 - RM) / (ese2 + RM);
    sinthe = -sqrt(1.0 - costh);
    costhe = sqrt(costh);
    uphi32(tk, &up, costhe, sinthe);
}

/* bhabha (ompmc.c:4438-4525). */
static void bhabha(track_t *tk) {
    const omc_tables *t = tk->c->t;
    const omc_regions *rg = tk->c->rg;
    int np = tk->np;
    int irl = tk->ir[np];
    int imed = rg->med[irl];
    double eip = tk->e[np];
    double ekin = eip - RM;
    double t0 = ekin / RM;
    double e0 = t0 + 1.0;
    double yy = 1.0 / (t0 + 2.0);
    double beta2 = (pow(e0, 2.0) - 1.0) / pow(e0, 2.0);
    double ep0 = t->te[imed] / ekin;
    double ep0c = 1.0 - ep0;
    double yp = 1.0 - 2.0 * yy;
    tk->npold = np;
    double b1, b2, b3, b4;
    b4 = pow(yp, 3.0);
    b3 = b4 + pow(yp, 2.0);
    b2 = yp * (3.0 + pow(yy, 2.0));
    b1 = 2.0 - pow(yy, 2.0);
    double rnno03, rnno04, br, rejf2;
    do {
        rnno03 = rnd(tk);
        br = ep0 / (1.0 - ep0c * rnno03);
        rnno04 = rnd(tk);
        rejf2 = (1.0 - beta2 * br * (b1 - br * (b2 - br * (b3 - br * b4))));
    } while (rnno04 > rejf2);
    if (br < 0.5) {
        tk->iq[np + 1] = -1;
    } else {
        tk->iq[np] = -1;
        tk->iq[np + 1] = 1;
        br = 1.0 - br;
    }
    br = fmax(br, 0.0);
    double ekse2 = br * ekin;
    double ese1 = eip - ekse2;
    double ese2 = ekse2 + RM;
    tk->e[np] = ese1;
    tk->e[np + 1] = ese2;
    double h1 = (eip + RM) / ekin;
    double costh = fmin(1.0, h1 * (ese1 - RM) / (ese1 + RM));
    double sinthe = sqrt(1.0 - costh);
    double costhe = sqrt(costh);
    uphi_t up;
    uphi21(tk, &up, costhe, sinthe);
    np += 1;
    tk->np = np;
    costh = h1 * (ese2 - RM) / (ese2 + RM);
    sinthe = -sqrt(1.0 - costh);
    costhe = sqrt(costh);
    uphi32(tk, &up, costhe, sinthe);
}

/* annih (ompmc.c:4528-4645): two-photon annihilation in flight. */
static void annih(track_t *tk) {
    int np = tk->np;
    double avip = tk->e[np] + RM;
    double a = avip / RM;
    double g, tt, p;
    g = a - 1.0;
    tt = g - 1.0;
    p = sqrt(a * tt);
    tk->npold = np;
    double pot = p / tt;
    double ep0 = 1.0 / (a + p);
    double wsamp = log((1.0 - ep0) / ep0);
    double aa = tk->u[np], bb = tk->v[np], cc = tk->w[np];
    double sinpsi = pow(aa, 2.0) + pow(bb, 2.0);
    double sindel = 0.0, cosdel = 0.0;
    if (sinpsi > 1.0E-20) {
        sinpsi = sqrt(sinpsi);
        sindel = bb / sinpsi;
        cosdel = aa / sinpsi;
    }
    double ep, rejf, rnno01, rnno02;
    do {
        rnno01 = rnd(tk);
        ep = ep0 * exp(rnno01 * wsamp);
        rnno02 = rnd(tk);
        rejf = 1.0 - pow(ep * a - 1.0, 2.0) / (ep * (pow(a, 2.0) - 2.0));
    } while (rnno02 > rejf);
    double esg1 = avip * ep;
    tk->e[np] = esg1;
    tk->iq[np] = 0;
    double costhe = fmin(1.0, (esg1 - RM) * pot / esg1);
    double sinthe = sqrt(1.0 - pow(costhe, 2.0));
    double sphi, cphi;
    azimuth(tk, &cphi, &sphi);
    double us, vs;
    if (sinpsi >= 1.0E-10) {
        us = sinthe * cphi;
        vs = sinthe * sphi;
        tk->u[np] = cc * cosdel * us - sindel * vs + aa * costhe;
        tk->v[np] = cc * sindel * us + cosdel * vs + bb * costhe;
        tk->w[np] = cc * costhe - sinpsi * us;
    } else {
        tk->u[np] = sinthe * cphi;
        tk->v[np] = sinthe * sphi;
        tk->w[np] = cc * costhe;
    }
    np += 1;
    double esg2 = avip - esg1;
    tk->e[np] = esg2;
    tk->iq[np] = 0;
    transfer(tk, np, np - 1);
    costhe = fmin(1.0, (esg2 - RM) * pot / esg2);
    sinthe = -sqrt(1.0 - pow(costhe, 2.0));
    if (sinpsi >= 1.0E-10) {
        us = sinthe * cphi;
        vs = sinthe * sphi;
        tk->u[np] = cc * cosdel * us - sindel * vs + aa * costhe;
        tk->v[np] = cc * sindel * us + cosdel * vs + bb * costhe;
        tk->w[np] = cc * costhe - sinpsi * us;
    } else {
        tk->u[np] = sinthe * cphi;
        tk->v[np] = sinthe * sphi;
        tk->w[np] = cc * costhe;
    }
    tk->np = np;
    roulette_photons(tk, 0);
}

/* Energy deposit of a particle that stops here, with annihilation photons
 * for positrons (ompmc.c:4665-4686 and the same block at :5063-5087,
 * :5120-5141, :5262-5325).  Returns after the stack has been updated. */
static void terminate_charged(track_t *tk, int iq, double eie, double edep) {
    ausgab(tk, edep);
    if (iq > 0 && edep < eie) {
        rannih(tk);
        return;
    }
    tk->np -= 1;
}

/* electron (ompmc.c:4648-5433).  The loop structure is the reference's,
 * including the path-length bookkeeping that restarts at zero in every
 * ustep iteration (ompmc.c:4787). */
static void electron(track_t *tk) {
    const omc_tables *t = tk->c->t;
    const omc_regions *rg = tk->c->rg;
    int nmed = t->nmed;
    int np = tk->np;
    int irl = tk->ir[np];
    int imed = rg->med[irl];
    double rhof = rg->rhof[irl];
    double edep = 0.0;
    uphi_t up;
    double eie = tk->e[np];
    int iq = tk->iq[np];
    int qel = (1 + iq) / 2;
    int medold = imed;
    double rnno;
    if (eie <= rg->ecut[irl]) {
        edep = tk->e[np] - RM;
        terminate_charged(tk, iq, eie, edep);
        return;
    }
    double elke = 0.0;
    int lelke = 0;
    double sigratio = 0.0, rfict = 0.0;
    do {
        int compute_tstep = 1;
        double eke = eie - RM;
        double demfp = 0.0, sigf, sig0 = 0.0, dedx0, ustep = 0.0;
        if (imed != -1) {
            rnno = rnd(tk);
            if (rnno == 0.0) rnno = 1.0E-30;
            demfp = fmax(-log(rnno), EPSEMFP);
            elke = log(eke);
            lelke = pwlf_index(t->eke1, t->eke0, imed, elke) - 1;
            int ix = imed * MXEKE + lelke;
            if (t->sig_ismonotone[qel * nmed + imed]) {
                if (iq < 0) {
                    sig0 = pwlf(t->esig1, t->esig0, ix, elke);
                    dedx0 = pwlf(t->ededx1, t->ededx0, ix, elke);
                    sig0 /= dedx0;
                } else {
                    sig0 = pwlf(t->psig1, t->psig0, ix, elke);
                    dedx0 = pwlf(t->pdedx1, t->pdedx0, ix, elke);
                    sig0 /= dedx0;
                }
            } else {
                sig0 = (iq < 0) ? t->esig_e[imed] : t->psig_e[imed];
            }
        }
        do {
            int call_howfar = 0, do_single = 0, called_msdist = 0;
            double tstep, tustep, total_de, ekef, ekei, elkei, tuss;
            double total_tstep = 0.0;
            double range = 0.0, p2, beta2, etap, tvstep = 0.0, de = 0.0;
            double x_final = 0, y_final = 0, z_final = 0, u_final = 0, v_final = 0, w_final = 0;
            const double *rng_ep = t->range_ep + (size_t)qel * nmed * MXEKE + (size_t)(imed < 0 ? 0 : imed) * MXEKE;
            if (imed == -1) {
                tstep = 10.0E8;
                ustep = tstep;
                tustep = ustep;
                call_howfar = 1;
            } else {
                rhof = rg->rhof[irl];
                if (sig0 <= 0.0) {
                    tstep = 10.0E8;
                    sig0 = 1.0E-15;
                } else {
                    if (compute_tstep) {
                        total_de = demfp / sig0;
                        ekef = eke - total_de;
                        if (ekef <= t->e_array[imed * MXEKE + 0]) {
                            tstep = 10.0E8;
                        } else {
                            double elkef = log(ekef);
                            int lelkef = pwlf_index(t->eke1, t->eke0, imed, elkef) - 1;
                            if (lelkef == lelke) {
                                tstep = drange(t, imed, iq, lelke, eke, ekef, elke, elkef);
                            } else {
                                ekei = t->e_array[imed * MXEKE + lelke];
                                elkei = (lelke + 1 - t->eke0[imed]) / t->eke1[imed];
                                tuss = drange(t, imed, iq, lelke, eke, ekei, elke, elkei);
                                ekei = t->e_array[imed * MXEKE + lelkef + 1];
                                elkei = ((lelkef + 2) - t->eke0[imed]) / t->eke1[imed];
                                tstep = drange(t, imed, iq, lelkef, ekei, ekef, elkei, elkef);
                                tstep += tuss + rng_ep[lelke] - rng_ep[lelkef + 1];
                            }
                        }
                        total_tstep = tstep;
                        compute_tstep = 0;
                    }
                    tstep = total_tstep / rhof;
                }
                int ix = imed * MXEKE + lelke;
                dedx0 = (iq < 0) ? pwlf(t->ededx1, t->ededx0, ix, elke) : pwlf(t->pdedx1, t->pdedx0, ix, elke);
                double dedx = rhof * dedx0;
                double tmxs = pwlf(t->tmxs1, t->tmxs0, ix, elke);
                tmxs /= rhof;
                ekei = t->e_array[imed * MXEKE + lelke];
                elkei = (lelke + 1 - t->eke0[imed]) / t->eke1[imed];
                range = drange(t, imed, iq, lelke, eke, ekei, elke, elkei);
                range += rng_ep[lelke];
                range /= rhof;
                tustep = fmin(fmin(tstep, tmxs), range);
                double tperp = hownear(tk);
                tk->dnear[np] = tperp;
                double blccl = rhof * t->blcc[imed];
                double xccl = rhof * t->xcc[imed];
                p2 = eke * (eke + 2.0 * RM);
                beta2 = p2 / (p2 + pow(RM, 2.0));
                etap = (iq < 0) ? pwlf(t->etae_ms1, t->etae_ms0, ix, elke) : pwlf(t->etap_ms1, t->etap_ms0, ix, elke);
                double ms_corr = pwlf(t->blcce1, t->blcce0, ix, elke);
                blccl = blccl / etap / (1.0 + 0.25 * etap * xccl / blccl / p2) * ms_corr;
                double ssmfp = beta2 / blccl;
                double skindepth = SKIN_DEPTH_FOR_BCA * ssmfp;
                tustep = fmin(tustep, fmax(tperp, skindepth));
                if ((tustep <= tperp) && (tustep > skindepth)) {
                    call_howfar = 0;
                    do_single = 0;
                    called_msdist = 1;
                    de = eloss(t, imed, iq, rhof, tustep, range, eke, elke, lelke);
                    tvstep = tustep;
                    ustep = msdist(tk, imed, iq, rhof, de, tustep, eke, &x_final, &y_final, &z_final, &u_final,
                                   &v_final, &w_final);
                } else {
                    called_msdist = 0;
                    rnno = rnd(tk);
                    if (rnno < 1.0E-30) rnno = 1.0E-30;
                    double lambda = (-1.0) * log(1.0 - rnno);
                    double lambda_max = 0.5 * blccl * RM / dedx;
                    lambda_max *= (eke / RM + 1.0) * (eke / RM + 1.0) * (eke / RM + 1.0);
                    if (lambda >= 0.0 && lambda_max > 0.0) {
                        if (lambda < lambda_max) tuss = lambda * ssmfp * (1.0 - 0.5 * lambda / lambda_max);
                        else tuss = 0.5 * lambda * ssmfp;
                        if (tuss < tustep) {
                            tustep = tuss;
                            do_single = 1;
                        } else {
                            do_single = 0;
                        }
                    } else {
                        tk->np -= 1;
                        return;
                    }
                    ustep = tustep;
                    call_howfar = (ustep < tperp) ? 0 : 1;
                }
            }
            int irold = tk->ir[np];
            int irnew = tk->ir[np];
            int idisc = 0;
            if (call_howfar) howfar(tk, &idisc, &irnew, &ustep);
            if (idisc > 0) {
                edep = (iq > 0) ? tk->e[np] + RM : tk->e[np] - RM;
                terminate_charged(tk, iq, eie, edep);
                return;
            }
            if (ustep < 0) ustep = 0.0;
            double vstep;
            if (ustep == 0.0f || imed == -1) {
                if (ustep != 0.0f) {
                    vstep = ustep;
                    tvstep = vstep;
                    tk->x[np] += tk->u[np] * vstep;
                    tk->y[np] += tk->v[np] * vstep;
                    tk->z[np] += tk->w[np] * vstep;
                    tk->dnear[np] -= vstep;
                }
                if (irnew != irold) {
                    tk->ir[np] = irnew;
                    irl = irnew;
                    imed = rg->med[irl];
                }
                if (eie <= rg->ecut[irl]) {
                    edep = tk->e[np] - RM;
                    terminate_charged(tk, iq, eie, edep);
                    return;
                }
                break;
            }
            vstep = ustep;
            if (call_howfar) {
                tvstep = vstep;
                if (tvstep != tustep) do_single = 0;
                de = eloss(t, imed, iq, rhof, tvstep, range, eke, elke, lelke);
            } else {
                tvstep = tustep;
                if (called_msdist == 0) de = eloss(t, imed, iq, rhof, tvstep, range, eke, elke, lelke);
            }
            edep = de;
            ekef = eke - de;
            double sinthe, costhe;
            if (called_msdist == 0) {
                if (do_single) {
                    double ekems = fmax(ekef, rg->ecut[irl] - RM);
                    p2 = ekems * (ekems + 2.0 * RM);
                    beta2 = p2 / (p2 + pow(RM, 2.0));
                    double chia2 = t->xcc[imed] / (4.0 * t->blcc[imed] * p2);
                    double elkems = log(ekems);
                    int lelkems = pwlf_index(t->eke1, t->eke0, imed, elkems) - 1;
                    int jx = MXEKE * imed + lelkems;
                    etap = (iq < 0) ? pwlf(t->etae_ms1, t->etae_ms0, jx, elkems)
                                    : pwlf(t->etap_ms1, t->etap_ms0, jx, elkems);
                    chia2 *= etap;
                    sscat(tk, imed, qel, chia2, elkems, beta2, &costhe, &sinthe);
                } else {
                    sinthe = 0.0f;
                    costhe = 1.0f;
                }
            }
            if (called_msdist == 0) {
                x_final = tk->x[np] + tk->u[np] * vstep;
                y_final = tk->y[np] + tk->v[np] * vstep;
                z_final = tk->z[np] + tk->w[np] * vstep;
                if (do_single) uphi21(tk, &up, costhe, sinthe);
                u_final = tk->u[np];
                v_final = tk->v[np];
                w_final = tk->w[np];
            }
            ausgab(tk, edep);
            tk->x[np] = x_final;
            tk->y[np] = y_final;
            tk->z[np] = z_final;
            tk->u[np] = u_final;
            tk->v[np] = v_final;
            tk->w[np] = w_final;
            tk->dnear[np] -= vstep;
            irold = tk->ir[np];
            eie -= edep;
            tk->e[np] = eie;
            if (irnew == irl && eie <= rg->ecut[irl]) {
                edep = tk->e[np] - RM;
                terminate_charged(tk, iq, eie, edep);
                return;
            }
            medold = imed;
            if (imed != -1) {
                eke = eie - RM;
                elke = log(eke);
                lelke = pwlf_index(t->eke1, t->eke0, imed, elke) - 1;
            }
            if (irnew != irold) {
                tk->ir[np] = irnew;
                irl = irnew;
                imed = rg->med[irl];
            }
            if (eie <= rg->ecut[irl]) {
                edep = tk->e[np] - RM;
                terminate_charged(tk, iq, eie, edep);
                return;
            }
            if (imed != medold) break;
            demfp -= de * sig0;
            total_de -= de;
            total_tstep -= tvstep * rhof;
            if (total_tstep < 1.0E-9) demfp = 0.0;
        } while (demfp >= EPSEMFP);
        if ((imed != medold) || (ustep == 0.0) || (imed == -1)) continue;
        int ix = imed * MXEKE + lelke;
        if (iq < 0) {
            sigf = pwlf(t->esig1, t->esig0, ix, elke);
            dedx0 = pwlf(t->ededx1, t->ededx0, ix, elke);
            sigf /= dedx0;
        } else {
            sigf = pwlf(t->psig1, t->psig0, ix, elke);
            dedx0 = pwlf(t->pdedx1, t->pdedx0, ix, elke);
            sigf /= dedx0;
        }
        sigratio = sigf / sig0;
        rfict = rnd(tk);
    } while (rfict >= sigratio);
    int ix = imed * MXEKE + lelke;
    if (iq < 0) {
        double ebr1 = pwlf(t->ebr11, t->ebr10, ix, elke);
        rnno = rnd(tk);
        if (rnno <= ebr1) {
            brems(tk);
        } else {
            if (tk->e[np] <= t->thmoll[imed]) {
                if (ebr1 <= 0) return;
                brems(tk);
            } else {
                moller(tk);
            }
        }
    } else {
        double pbr1 = pwlf(t->pbr11, t->pbr10, ix, elke);
        rnno = rnd(tk);
        if (rnno < pbr1) {
            brems(tk);
        } else {
            double pbr2 = pwlf(t->pbr21, t->pbr20, ix, elke);
            if (rnno < pbr2) bhabha(tk);
            else annih(tk);
        }
    }
}

/* initHistory (omc_dosxyz.c:964-1068). */
static void init_history(track_t *tk) {
    const omc_source *s = tk->c->src;
    const omc_phantom *g = tk->c->ph;
    tk->np = 0;
    tk->iq[0] = s->charge;
    double ein;
    if (s->spectrum) {
        double rnno1 = rnd(tk);
        double rnno2 = rnd(tk);
        int k = (int)fmin(s->deltak * rnno1, s->deltak - 1.0);
        ein = s->cdfinv1[k] + rnno2 * s->cdfinv2[k];
    } else {
        ein = s->energy;
    }
    tk->e[0] = (tk->iq[0] != 0) ? ein + RM : ein;
    tk->ensrc += ein;
    double rxyz;
    if (s->xsize == 0.0 || s->ysize == 0.0) {
        tk->x[0] = s->xinl;
        tk->y[0] = s->yinl;
        rxyz = sqrt(pow(s->ssd, 2.0) + pow(tk->x[0], 2.0) + pow(tk->y[0], 2.0));
        tk->w[0] = s->ssd / rxyz;
    } else {
        double fw, rnno3;
        do {
            rnno3 = rnd(tk);
            tk->x[0] = rnno3 * s->xsize + s->xinl;
            rnno3 = rnd(tk);
            tk->y[0] = rnno3 * s->ysize + s->yinl;
            rnno3 = rnd(tk);
            rxyz = sqrt(s->ssd * s->ssd + tk->x[0] * tk->x[0] + tk->y[0] * tk->y[0]);
            tk->w[0] = s->ssd / rxyz;
            fw = tk->w[0] * tk->w[0] * tk->w[0];
        } while (rnno3 >= fw);
    }
    tk->z[0] = g->zbounds[0];
    tk->u[0] = tk->x[0] / rxyz;
    tk->v[0] = tk->y[0] / rxyz;
    int ix, iy;
    if (s->xsize == 0.0) {
        ix = s->ixinl;
    } else {
        ix = s->ixinl - 1;
        while ((g->xbounds[ix + 1] < tk->x[0]) && ix < g->nx - 1) ix++;
    }
    if (s->ysize == 0.0) {
        iy = s->iyinl;
    } else {
        iy = s->iyinl - 1;
        while ((g->ybounds[iy + 1] < tk->y[0]) && iy < g->ny - 1) iy++;
    }
    tk->ir[0] = 1 + ix + iy * g->nx;
    tk->wt[0] = 1.0;
    tk->dnear[0] = 0.0;
}

/* shower (ompmc.c:5436-5447). */
static void shower(track_t *tk) {
    while (tk->np >= 0) {
        if (tk->iq[tk->np] == 0) photon(tk);
        else electron(tk);
    }
}

/* Energy deposited inside the phantom (regions >= 1) by each batch of the
 * last omc_oracle_run, for the batch uncertainty of the total. */
#define ORACLE_MAX_BATCHES 65536
static double g_batch_etot[ORACLE_MAX_BATCHES];
static int g_batch_n;

int omc_oracle_batch_totals(double *out, int cap) {
    int n = g_batch_n < cap ? g_batch_n : cap;
    for (int i = 0; i < n; i++) out[i] = g_batch_etot[i];
    return n;
}

int omc_oracle_run(const omc_tables *t, const omc_phantom *ph, const omc_regions *rg, const omc_source *src,
                   int nsplit, long long nperbatch, int nbatch, int ixx, int jxx, int nthreads, double *accum_endep,
                   double *accum_endep2, omc_oracle_result *res) {
    int nreg = rg->nreg;
    double *endep = calloc(nreg, sizeof(double));
    if (!endep) return 2;
    memset(accum_endep, 0, nreg * sizeof(double));
    memset(accum_endep2, 0, nreg * sizeof(double));
    ctx_t c = {t, ph, rg, src, nsplit < 1 ? 1 : nsplit, endep, NULL};
#ifdef _OPENMP
    if (nthreads <= 0) nthreads = omp_get_num_procs();
#else
    nthreads = 1;
#endif
    track_t **tks = calloc(nthreads, sizeof(track_t *));
    for (int i = 0; i < nthreads; i++) {
        tks[i] = calloc(1, sizeof(track_t));
        tks[i]->c = &c;
        ranmar_init(&tks[i]->rng, ixx, jxx + (nthreads > 1 ? i : 0));
    }
    int overflow = 0;
#ifdef _OPENMP
    double t0 = omp_get_wtime();
#endif
    for (int ib = 0; ib < nbatch; ib++) {
        if (nthreads > 1) {
            #pragma omp parallel for schedule(dynamic) num_threads(nthreads)
            for (long long ih = 0; ih < nperbatch; ih++) {
#ifdef _OPENMP
                track_t *tk = tks[omp_get_thread_num()];
#else
                track_t *tk = tks[0];
#endif
                init_history(tk);
                shower(tk);
            }
        } else {
            for (long long ih = 0; ih < nperbatch; ih++) {
                init_history(tks[0]);
                shower(tks[0]);
            }
        }
        double etot = 0.0;
        for (int r = 0; r < nreg; r++) {
            double e = endep[r];
            accum_endep[r] += e;
            accum_endep2[r] += e * e;
            if (r > 0) etot += e;
        }
        if (ib < ORACLE_MAX_BATCHES) g_batch_etot[ib] = etot;
        memset(endep, 0, nreg * sizeof(double));
    }
    g_batch_n = nbatch < ORACLE_MAX_BATCHES ? nbatch : ORACLE_MAX_BATCHES;
    double ens = 0.0;
    for (int i = 0; i < nthreads; i++) {
        ens += tks[i]->ensrc;
        overflow |= tks[i]->overflow;
        free(tks[i]);
    }
    free(tks);
    free(endep);
    if (res) {
        res->ensrc = ens;
#ifdef _OPENMP
        res->seconds = omp_get_wtime() - t0;
#else
        res->seconds = 0.0;
#endif
        res->histories = nperbatch * nbatch;
        res->nthreads = nthreads;
        res->status = overflow;
    }
    return overflow;
}

/* ---------------------------------------------------------------------- */
/* omc_matrad: beamlet source and dose-influence matrix.                    */

/* initHistory(ibeamlet) (ucodes/omc_matrad/omc_matrad.c:1084-1254): energy
 * as in omc_dosxyz, a uniform point on the beamlet's bixel, moved back
 * along the line to its beam's source point onto the phantom surface, and
 * the voxel found by linear scans.  The reference clamps z against
 * ybounds[0] (:1225); that is kept. */
static void init_beamlet_history(track_t *tk, int ib) {
    const omc_source *s = tk->c->src;
    const omc_beamlets *b = tk->c->bl;
    const omc_phantom *g = tk->c->ph;
    tk->np = 0;
    tk->iq[0] = s->charge;
    double ein;
    if (s->spectrum) {
        double rnno1 = rnd(tk);
        double rnno2 = rnd(tk);
        int k = (int)fmin(s->deltak * rnno1, s->deltak - 1.0);
        ein = s->cdfinv1[k] + rnno2 * s->cdfinv2[k];
    } else {
        ein = s->energy;
    }
    tk->e[0] = (tk->iq[0] != 0) ? ein + RM : ein;
    tk->ensrc += ein;
    double rnno1 = rnd(tk);
    double rnno2 = rnd(tk);
    double xiso = rnno1 * b->xside1[ib] + rnno2 * b->xside2[ib] + b->xcorner[ib];
    double yiso = rnno1 * b->yside1[ib] + rnno2 * b->yside2[ib] + b->ycorner[ib];
    double ziso = rnno1 * b->zside1[ib] + rnno2 * b->zside2[ib] + b->zcorner[ib];
    int ibeam = b->ibeam[ib];
    double vnorm = sqrt(pow(xiso - b->xsource[ibeam], 2.0) + pow(yiso - b->ysource[ibeam], 2.0) +
                        pow(ziso - b->zsource[ibeam], 2.0));
    double u = -(xiso - b->xsource[ibeam]) / vnorm;
    double v = -(yiso - b->ysource[ibeam]) / vnorm;
    double w = -(ziso - b->zsource[ibeam]) / vnorm;
    double ustep = 1.0E5, dist;
    if (u > 0.0) {
        dist = (g->xbounds[g->nx] - xiso) / u;
        if (dist < ustep) ustep = dist;
    }
    if (u < 0.0) {
        dist = -(xiso - g->xbounds[0]) / u;
        if (dist < ustep) ustep = dist;
    }
    if (v > 0.0) {
        dist = (g->ybounds[g->ny] - yiso) / v;
        if (dist < ustep) ustep = dist;
    }
    if (v < 0.0) {
        dist = -(yiso - g->ybounds[0]) / v;
        if (dist < ustep) ustep = dist;
    }
    if (w > 0.0) {
        dist = (g->zbounds[g->nz] - ziso) / w;
        if (dist < ustep) ustep = dist;
    }
    if (w < 0.0) {
        dist = -(ziso - g->zbounds[0]) / w;
        if (dist < ustep) ustep = dist;
    }
    double x = xiso + ustep * u, y = yiso + ustep * v, z = ziso + ustep * w;
    tk->u[0] = -u;
    tk->v[0] = -v;
    tk->w[0] = -w;
    if (x < g->xbounds[0]) x = g->xbounds[0] + 2.0 * DBL_MIN;
    if (x > g->xbounds[g->nx]) x = g->xbounds[g->nx] - 2.0 * DBL_MIN;
    if (y < g->ybounds[0]) y = g->ybounds[0] + 2.0 * DBL_MIN;
    if (y > g->ybounds[g->ny]) y = g->ybounds[g->ny] - 2.0 * DBL_MIN;
    if (z < g->zbounds[0]) z = g->ybounds[0] + 2.0 * DBL_MIN;
    if (z > g->zbounds[g->nz]) z = g->zbounds[g->nz] - 2.0 * DBL_MIN;
    tk->x[0] = x;
    tk->y[0] = y;
    tk->z[0] = z;
    int ix = 0, iy = 0, iz = 0;
    while (g->xbounds[ix + 1] < x) ix++;
    while (g->ybounds[iy + 1] < y) iy++;
    while (g->zbounds[iz + 1] < z) iz++;
    tk->ir[0] = 1 + ix + iy * g->nx + iz * g->nx * g->ny;
    tk->wt[0] = 1.0;
    tk->dnear[0] = 0.0;
}

/* Dose of one beamlet from its batch sums, then threshold and column of
 * the CSC matrix (omc_matrad.c:839-919 accumulateResults with iout = 1,
 * :1426-1482 threshold and column fill). */
static int dij_column(const omc_phantom *ph, const double *accum, long long nhist, int nbatch, double rel,
                      double *dose, omc_dij *d, long long *cap, int col) {
    int nx = ph->nx, ny = ph->ny, nz = ph->nz;
    long long nvox = (long long)nx * ny * nz;
    double inc_fluence = (double)nhist;
    for (int iz = 0; iz < nz; iz++)
        for (int iy = 0; iy < ny; iy++)
            for (int ix = 0; ix < nx; ix++) {
                long long irl = 1 + ix + (long long)iy * nx + (long long)iz * nx * ny;
                double endep = accum[irl] / (double)nbatch;
                if (endep == 0.0) endep = 0.0;
                double mass = (ph->xbounds[ix + 1] - ph->xbounds[ix]) * (ph->ybounds[iy + 1] - ph->ybounds[iy]) *
                              (ph->zbounds[iz + 1] - ph->zbounds[iz]);
                mass *= ph->density[irl - 1];
                endep *= 1.602E-10 / (mass * inc_fluence);
                if (ph->density[irl - 1] < 0.044) endep = 0.0;
                dose[irl] = endep;
            }
    double dmax = 0.0;
    for (long long irl = 1; irl < nvox + 1; irl++)
        if (dose[irl] > dmax) dmax = dose[irl];
    double thresh = dmax * rel;
    long long nnz = 0;
    for (long long irl = 1; irl < nvox + 1; irl++)
        if (dose[irl] > thresh) nnz++;
    if (d->nnz + nnz > *cap) {
        long long nc = (d->nnz + nnz) * 2 + 16;
        int *ri = realloc(d->row_idx, nc * sizeof(int));
        double *va = realloc(d->values, nc * sizeof(double));
        if (!ri || !va) return 2;
        d->row_idx = ri;
        d->values = va;
        *cap = nc;
    }
    for (long long irl = 1; irl < nvox + 1; irl++)
        if (dose[irl] > thresh) {
            d->row_idx[d->nnz] = (int)(irl - 1);
            d->values[d->nnz] = dose[irl];
            d->nnz++;
        }
    d->col_ptr[col + 1] = d->nnz;
    return 0;
}

int omc_oracle_run_dij(const omc_tables *t, const omc_phantom *ph, const omc_regions *rg, const omc_source *src,
                       const omc_beamlets *bl, int nsplit, const long long *nhist, long long nperbatch, int nbatch,
                       int ixx, int jxx, int nthreads, double rel_threshold, omc_dij *out, omc_oracle_result *res) {
    int nreg = rg->nreg;
    memset(out, 0, sizeof *out);
    out->nrows = nreg - 1;
    out->ncols = bl->nbeamlets;
    out->col_ptr = calloc((size_t)bl->nbeamlets + 1, sizeof(long long));
    double *endep = calloc(nreg, sizeof(double));
    double *accum = calloc(nreg, sizeof(double));
    double *dose = calloc(nreg, sizeof(double));
    if (!endep || !accum || !dose || !out->col_ptr) return 2;
    ctx_t c = {t, ph, rg, src, nsplit < 1 ? 1 : nsplit, endep, bl};
#ifdef _OPENMP
    if (nthreads <= 0) nthreads = omp_get_num_procs();
#else
    nthreads = 1;
#endif
    track_t **tks = calloc(nthreads, sizeof(track_t *));
    for (int i = 0; i < nthreads; i++) {
        tks[i] = calloc(1, sizeof(track_t));
        tks[i]->c = &c;
        ranmar_init(&tks[i]->rng, ixx, jxx + (nthreads > 1 ? i : 0));
    }
#ifdef _OPENMP
    double t0 = omp_get_wtime();
#endif
    long long cap = 0, total = 0;
    int status = 0;
    for (int ib = 0; ib < bl->nbeamlets && !status; ib++) {
        /* Histories of this beamlet: nbatch batches of nhist/nbatch
         * (omc_matrad.c:1321-1335 and the loop at :1389-1404). */
        long long nb = nhist ? nhist[ib] : nperbatch * nbatch;
        long long per = nb / nbatch;
        if (per == 0) per = 1;
        for (int batch = 0; batch < nbatch; batch++) {
            if (nthreads > 1) {
                #pragma omp parallel for schedule(dynamic) num_threads(nthreads)
                for (long long ih = 0; ih < per; ih++) {
#ifdef _OPENMP
                    track_t *tk = tks[omp_get_thread_num()];
#else
                    track_t *tk = tks[0];
#endif
                    init_beamlet_history(tk, ib);
                    shower(tk);
                }
            } else {
                for (long long ih = 0; ih < per; ih++) {
                    init_beamlet_history(tks[0], ib);
                    shower(tks[0]);
                }
            }
            for (int r = 0; r < nreg; r++) accum[r] += endep[r];
            memset(endep, 0, nreg * sizeof(double));
        }
        total += per * nbatch;
        status = dij_column(ph, accum, per * nbatch, nbatch, rel_threshold, dose, out, &cap, ib);
        memset(accum, 0, nreg * sizeof(double));
    }
    double ens = 0.0;
    int overflow = 0;
    for (int i = 0; i < nthreads; i++) {
        ens += tks[i]->ensrc;
        overflow |= tks[i]->overflow;
        free(tks[i]);
    }
    free(tks);
    free(endep);
    free(accum);
    free(dose);
    if (res) {
        res->ensrc = ens;
#ifdef _OPENMP
        res->seconds = omp_get_wtime() - t0;
#else
        res->seconds = 0.0;
#endif
        res->histories = total;
        res->nthreads = nthreads;
        res->status = overflow;
    }
    return status ? status : overflow;
}

void omc_oracle_dij_free(omc_dij *d) {
    if (!d) return;
    free(d->col_ptr);
    free(d->row_idx);
    free(d->values);
    memset(d, 0, sizeof *d);
}
