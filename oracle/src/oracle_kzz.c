/*
 * ORACLE -- test infrastructure, not the product.  Calc_Kzz per column, scalar C in the
 * reference's evaluation order: pydyn diffusion.py:76-89 (ustar), :92-104 (geopotential),
 * :107-110 (mass_t), :113-120 (_winds), :123-152 (_pbl_pass), :155-253 (bldiff), :256-263 (dkg),
 * :266-276 (calc_kzz).  exp / log / pow / cos are the package's gbmath, the functions pydyn is
 * pointed at through its ops.use_libm hook when the golden fixtures are made; cube is (x x) x.
 * jqif(x, y) = 1 where x - y has a clear sign bit.
 */
#include <math.h>

#include "../../pydyn_gb300/csrc/gbmath.h"
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

typedef struct {
    double *p;
    int64_t n[4];
    int64_t s[4];
} ov;

#define A2(v, i, j) ((v)->p[(int64_t)(i) * (v)->s[0] + (int64_t)(j) * (v)->s[1]])
#define A3(v, i, j, l) ((v)->p[(int64_t)(i) * (v)->s[0] + (int64_t)(j) * (v)->s[1] + (int64_t)(l) * (v)->s[2]])

static const double GRAV = 9.80665, PI_ = 3.14159265358979;
static const double AE = 6.371e6, VKARMAN = 0.4, CP_AIR = 1004.0, LVAP = 2.5e6, RGAS = 8.3144, XMAIR = 28.94;
static const double RHO_AIR = 1.2;
static const double CKMIN = 1.0e-15, SFFRAC = 0.1, APZERO = 100000.0, BETAH = 15.0, FAK = 8.5, FAKN = 7.2;
static const double TINY = 1.0e-9, ZACB = 100.0, RICR = 0.3, SSFRAC = 0.1, KVHMIN = 0.1;

static double jqif(double x, double y) { return signbit(x - y) ? 0.0 : 1.0; }
static double npmax(double a, double b) { return isnan(a) ? a : (isnan(b) ? b : (a > b ? a : b)); }
static double npmin(double a, double b) { return isnan(a) ? a : (isnan(b) ? b : (a < b ? a : b)); }
static double cube(double x) { return (x * x) * x; }

/* One column's pblh sweep (diffusion.py:123-152). */
static double pbl_pass(double pblh, const double *whm, const double *uw, const double *vw, const double *wthm,
                       const double *q, double ustr, double wtseff, double ref, int first, int lm) {
    const double zcrdq = 1.0 / (RGAS * 1.0e3 / XMAIR / 461.51) - 1.0;
    double jwork = 1.0, wrino = 0.0;
    for (int k = first ? 0 : 1; k < lm; k++) {
        double du = uw[k] - uw[0], dv = vw[k] - vw[0];
        double vvk = npmax(du * du + dv * dv + ZACB * ustr * ustr, TINY);
        double tkv = wthm[k] * (1.0 + zcrdq * q[k]);
        double dz = whm[k] - whm[0];
        double zrino = first ? GRAV * (tkv - wtseff) * dz / (wtseff * vvk) : GRAV * (tkv - ref) * dz / (vvk * wtseff);
        zrino = zrino + copysign(1.0e-10, zrino);
        zrino = jwork * zrino;
        double jq = jqif(RICR, zrino);
        double frac = (RICR - wrino) / (zrino - wrino);
        double at_ricr = k == 0 ? frac * whm[k] : whm[k - 1] + frac * (whm[k] - whm[k - 1]);
        pblh = jq * pblh + (1.0 - jq) * at_ricr;
        jwork = jq * jwork;
        wrino = zrino + (1.0 - jwork) * 0.1;
    }
    return first ? (1.0 - jwork) * pblh + whm[lm - 1] * jwork : (1.0 - jwork) * pblh + jwork * whm[lm - 1];
}

/* calc_kzz of a region: every argument as diffusion.calc_kzz takes it, surface fields in the
 * order oro, lsm, sr, srols, u10m, v10m, sshf, slhf, ewss, nsss (im, jm views); outputs dkg
 * (im, jm, lmax) and, if given, pblh (im, jm). */
void or_calc_kzz(const ov *spm, const ov *sp, const ov *pu, const ov *pv, const ov *t, const ov *q, const ov *surf,
                 const double *at, const double *bt, const double *dxyp, int lmax, double dx, double dy, double ybeg,
                 const ov *dkg, const ov *pblh_out) {
    const int im = (int)t->n[0], jm = (int)t->n[1], lm = (int)t->n[2];
    const double RAIR = RGAS * 1.0e3 / XMAIR, EPSILO = RAIR / 461.51, ZKAPPA = RAIR / CP_AIR;
    const double ZCRDQ = 1.0 / EPSILO - 1.0, ONET = 1.0 / 3.0, CCON = SFFRAC * VKARMAN, BINM = 15.0 * SFFRAC;
    const double GTOR = PI_ / 180.0;
    const ov *oro = &surf[0], *lsm = &surf[1], *sr = &surf[2], *srols = &surf[3], *u10m = &surf[4], *v10m = &surf[5];
    const ov *sshf = &surf[6], *slhf = &surf[7], *ewss = &surf[8], *nsss = &surf[9];
#pragma omp parallel
    {  /* columns are independent: each thread its own work arrays */
    double *w = malloc(sizeof(double) * (lm + 2) * 16);
    double *gph = w, *phlb = gph + (lm + 2), *m = phlb + (lm + 2), *pf = m + (lm + 2), *wthm = pf + (lm + 2);
    double *zthvk = wthm + (lm + 2), *whm = zthvk + (lm + 2), *uw = whm + (lm + 2), *vw = uw + (lm + 2);
    double *qc = vw + (lm + 2), *tc = qc + (lm + 2), *kvh = tc + (lm + 2), *logpf = kvh + (lm + 2);
#pragma omp for schedule(dynamic, 1)
    for (int j = 0; j < jm; j++) {
        const double lat = ybeg + 0.5 * dy + dy * j;
        const double dxx = AE * dx * GTOR * gbm_cos(lat * GTOR), dyy = AE * dy * GTOR;
        for (int i = 0; i < im; i++) {
            /* ustar */
            double xland = A2(lsm, i, j) / 100.0;
            double tau = sqrt(A2(ewss, i, j) * A2(ewss, i, j) + A2(nsss, i, j) * A2(nsss, i, j));
            double ustar_sea = npmax(0.001, sqrt(tau / RHO_AIR));
            double wind10m = sqrt(A2(u10m, i, j) * A2(u10m, i, j) + A2(v10m, i, j) * A2(v10m, i, j));
            double sr_land = npmax(1e-2, A2(srols, i, j));
            double sr_help = npmin(A2(sr, i, j), 0.03);
            double land = VKARMAN * wind10m / gbm_log(10.0 / sr_help) * gbm_log(75.0 / sr_help);
            land = land / gbm_log(10.0 / sr_land);
            double ustar_land = xland > 0.0 ? land : 0.0;
            double ustar_loc = xland * ustar_land + (1.0 - xland) * ustar_sea;
            /* geopotential of the interfaces (with sp), phlb and m (with spm) */
            const double s = A2(sp, i, j), sm = A2(spm, i, j);
            for (int l = 0; l < lm; l++) {
                tc[l] = A3(t, i, j, l);
                qc[l] = A3(q, i, j, l);
            }
            gph[0] = A2(oro, i, j) / GRAV;
            for (int k = 0; k < lm - 1; k++) {
                double tv = tc[k] * (1.0 + 0.608 * qc[k]);
                double pdown = at[k] + bt[k] * s, pup = at[k + 1] + bt[k + 1] * s;
                gph[k + 1] = gph[k] + tv * 287.05 * gbm_log(pdown / pup) / GRAV;
            }
            gph[lm] = 200000.0;
            for (int l = 0; l <= lm; l++) phlb[l] = at[l] + bt[l] * sm;
            for (int l = 0; l < lm; l++) m[l] = (phlb[l] - phlb[l + 1]) * dxyp[j] / GRAV;
            /* bldiff */
            const double z0 = gph[0];
            for (int l = 0; l < lm; l++) {
                pf[l] = (phlb[l] + phlb[l + 1]) * 0.5;
                wthm[l] = tc[l] * gbm_pow(APZERO / pf[l], ZKAPPA);
                zthvk[l] = wthm[l] * (1.0 + ZCRDQ * qc[l]);
                double intfac = (phlb[l] - pf[l]) / (phlb[l] - phlb[l + 1]);
                whm[l] = (gph[l] - z0) * (1.0 - intfac) + (gph[l + 1] - z0) * intfac;
                uw[l] = dxx * (A3(pu, i + 1, j, l) + A3(pu, i, j, l)) * 0.5 / m[l];
                vw[l] = dyy * (A3(pv, i, j + 1, l) + A3(pv, i, j, l)) * 0.5 / m[l];
                logpf[l] = gbm_log(pf[l]);
            }
            double dz1 = gph[1] - gph[0], dp1 = phlb[0] - phlb[1];
            double wheat = -A2(sshf, i, j) * dz1 * GRAV / dp1 / CP_AIR;
            double wqflx = -A2(slhf, i, j) * dz1 * GRAV / dp1 / LVAP;
            double ustr = npmax(ustar_loc, 0.01);
            double wtseff = wthm[0] * (1.0 + ZCRDQ * qc[0]);
            double wheatv = wheat + ZCRDQ * wthm[0] * wqflx;
            double wobkl = -wtseff * cube(ustr) / (GRAV * VKARMAN * (wheatv + copysign(1.0e-10, wheatv)));
            double pblh = pbl_pass(0.0, whm, uw, vw, wthm, qc, ustr, wtseff, 0.0, 1, lm);
            double jqh = jqif(wheatv, 0.0);
            double fmt0 = gbm_pow(jqh * (1.0 - BINM * pblh / wobkl) + (1.0 - jqh), ONET);
            double wsc0 = ustr * fmt0;
            double zexcess = wheatv * FAK / wsc0;
            double thvparc = wtseff + jqh * zexcess;
            pblh = pbl_pass(pblh, whm, uw, vw, wthm, qc, ustr, wtseff, thvparc, 0, lm);
            pblh = npmax(pblh, 100.0);
            if (pblh_out) A2(pblh_out, i, j) = pblh;
            const double P = pblh, W = wobkl, HV = wheatv, U = ustr, TS = wtseff;
            for (int k = 1; k < lm; k++) { /* interface k (between layers k-1 and k) */
                const double z = gph[k] - z0;
                /* free troposphere */
                double jq = jqif(1000.0, z);
                double zlambdac = jq * 300.0 + (1.0 - jq) * (30.0 + 270.0 * gbm_exp(1.0 - z / 1000.0));
                double cml2 = 1.0 / (1.0 / zlambdac + 1.0 / (VKARMAN * z));
                cml2 = cml2 * cml2;
                double du = uw[k] - uw[k - 1], dv = vw[k] - vw[k - 1];
                double zdup2 = npmax(du * du + dv * dv, 1.0e-10);
                double zdz = whm[k] - whm[k - 1];
                zdup2 = zdup2 / (zdz * zdz);
                double arg = (gbm_log(phlb[k]) - logpf[k - 1]) / (logpf[k] - logpf[k - 1]);
                double dthv = zthvk[k] - zthvk[k - 1];
                double zthva = zthvk[k - 1] + arg * dthv;
                double zsstab = GRAV / zthva * dthv / zdz;
                double zrinub = zsstab / zdup2;
                double zfunst = sqrt(npmax(1.0 - 18.0 * zrinub, 0.0));
                double zfstabh = 1.0 / (1.0 + 10.0 * zrinub * (1.0 + 8.0 * zrinub));
                double zkvn = cml2 * sqrt(zdup2);
                jq = jqif(zrinub, 0.0);
                double wkvf = jq * npmax(CKMIN, zkvn * zfstabh) + (1.0 - jq) * npmax(CKMIN, zkvn * zfunst);
                /* boundary layer */
                jq = jqif(P, z);
                double zh = jq * z / P;
                double zl = jq * z / W + (1.0 - jq);
                double zzh = jq * ((1.0 - zh) * (1.0 - zh));
                double jq1 = jqif(HV, 0.0);
                double jq2 = jq * (1.0 - jq1), jq3 = jq * jq1;
                double jq6 = jq1 * jqif(P, whm[k - 1]) * jqif(whm[k], P);
                jq1 = jqif(SFFRAC, zh);
                double jq4 = jq3 * jq1, jq5 = jq3 * (1.0 - jq1);
                cml2 = 1.0 / (1.0 / (VKARMAN * z) + 1.0 / 450.0);
                cml2 = cml2 * cml2;
                double jqq = jqif(zrinub, 0.0);
                zfstabh = jqq / (1.0 + 10.0 * zrinub * sqrt(1.0 + jqq * zrinub)) + (1.0 - jqq);
                double zpblk = cml2 * sqrt(zdup2) * zfstabh;
                double zkvh = jq2 * npmax(zpblk, KVHMIN) + (1.0 - jq2) * wkvf;
                double zslask = 1.0 - BETAH * zl;
                zslask = jq4 * zslask + (1.0 - jq4);
                zpblk = (1.0 - jq4) * zkvh + jq4 * (U * VKARMAN * z * zzh * gbm_pow(zslask, ONET));
                zslask = 1.0 - SSFRAC * BETAH * P / W;
                zslask = jq5 * zslask + (1.0 - jq5);
                double fmt = gbm_pow(zslask, ONET);
                double wsc = U * fmt;
                zpblk = (1.0 - jq5) * zpblk + jq5 * wsc * VKARMAN * z * zzh;
                double zwstr = gbm_pow(fabs(HV) * GRAV * P / TS, ONET);
                double obukov = jq3 * W - (1.0 - jq3);
                double stab = 1.0 - SSFRAC * BETAH * P / obukov;
                double term1 = gbm_pow(stab, ONET), term2 = sqrt(stab);
                double term3 = CCON * FAKN * zwstr / (U * term1);
                double pr = jq3 * (term1 / term2 + term3) + (1.0 - jq3);
                double kv = jq3 * npmax(zpblk / pr, KVHMIN) + (1.0 - jq3) * zkvh;
                double thvgrad = dthv / zdz;
                double kvhentr = 0.2 * HV / thvgrad;
                kvh[k - 1] = jq6 * kvhentr + (1.0 - jq6) * kv;
            }
            /* dkg across interfaces l+1, l < lmax - 1; zero at lmax - 1 */
            for (int l = 0; l < lmax; l++) {
                double v = 0.0;
                if (l < lmax - 1) {
                    double dz = gph[l + 2] - gph[l];
                    v = npmax(0.0, kvh[l]) * 2.0 * (m[l + 1] + m[l]) / (dz * dz);
                }
                A3(dkg, i, j, l) = v;
            }
        }
    }
    free(w);
    }
}
