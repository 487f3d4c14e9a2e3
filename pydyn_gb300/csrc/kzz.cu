// Calc_Kzz: the vertical diffusion exchange rate dkg of every column of a region.
//
// Eight launches, each with every lane on its own cell, column or interface (FP64 issue slots
// are GB300's scarcest resource, so no lane idles through another's serial work), the
// column-serial parts reduced to the recurrences that carry from level to level:
//   k_kzz_rows        thread per latitude: the zonal wind factor dxx (a cosine per row)
//   k_kzz_levels      thread per (column, level): potential temperature, the logarithms, the
//                     geopotential increments, the level winds -- into a work space
//   k_kzz_surface     thread per column: the geopotential's running sum, ustar, the surface
//                     fluxes and the Obukhov length
//   k_kzz_heights     thread per (column, level): the level height and the first
//                     bulk-Richardson sweep's level terms
//   k_kzz_sweep1      thread per column: the first sweep's running mask (pblh), the parcel excess
//   k_kzz_raw2        thread per (column, level): the second sweep's level terms
//   k_kzz_sweep2      thread per column: the second sweep (pblh) and the column constants of
//                     the diffusivity (w*, the Prandtl stability terms)
//   k_kzz_interfaces  thread per (column, interface), a warp 32 columns at one interface: the
//                     free-troposphere and boundary-layer diffusivities, then dkg of the
//                     interface (zero at lmax_conv - 1)
// Every value is the per-element statement of the reference in its order; exp / log / pow / cos
// are gbmath.h.  Reference: pydyn diffusion.py:71-276 (jqif, ustar, geopotential, mass_t,
// _winds, _pbl_pass, bldiff, dkg, calc_kzz).
#include "gb_common.cuh"
#include "gbmath.h"

namespace {

constexpr double GRAV = 9.80665, PI_ = 3.14159265358979, AE = 6.371e6, VKARMAN = 0.4, CP_AIR = 1004.0;
constexpr double LVAP = 2.5e6, RGAS = 8.3144, XMAIR = 28.94, RHO_AIR = 1.2, CKMIN = 1.0e-15, SFFRAC = 0.1;
constexpr double APZERO = 100000.0, BETAH = 15.0, FAK = 8.5, FAKN = 7.2, TINY = 1.0e-9, ZACB = 100.0;
constexpr double RICR = 0.3, SSFRAC = 0.1, KVHMIN = 0.1;
// z0, pblh, wobkl, wheatv, ustr, zwstr, t1a, t2a, t1b, t2b, wtseff, thvparc, then the interfaces'
// column constants: the Prandtl sums for jq3 = 0 and 1 and the reciprocal of the second, the free-convection
// stability 1 - SSFRAC BETAH pblh / wobkl and its cube root, the reciprocals of pblh and wobkl
constexpr int NCOLVAL = 19;
constexpr double RGRAV = 1.0 / GRAV;  // correctly rounded: the divisor's reciprocal for div_by_recip

struct KArgs {
    DV spm, sp, pu, pv, t, q, surf[10], dkg, pblh;
    const double *at, *bt, *dxyp;
    int im, jm, lm, lmax;
    double dx, dy, ybeg;
    // work space
    double *dxx, *wthm, *zthvk, *lpf, *lphlb, *dzg, *uw, *vw, *whm, *gph, *col;
    double *sw_vvk, *sw_dz, *sw_raw;  // the sweeps' level terms
};

__device__ __forceinline__ double S2(const DV &v, int i, int j) { return v.p[(int64_t)i * v.s0 + (int64_t)j * v.s1]; }
__device__ __forceinline__ double &S3(const DV &v, int i, int j, int l) {
    return v.p[(int64_t)i * v.s0 + (int64_t)j * v.s1 + (int64_t)l * v.s2];
}
// jqif(x, y) = nint(0.5 + sign(0.5, x - y)): 1 where x - y has a clear sign bit
__device__ __forceinline__ double jqif(double x, double y) { return signbit(x - y) ? 0.0 : 1.0; }
// the interfaces' free-convection blend as the reference writes it, for non-finite operands
static __device__ __noinline__ double zpblk_jq5_fp64(double jq5, double zpblk, double wsc, double z, double zzh) {
    return (1.0 - jq5) * zpblk + jq5 * wsc * VKARMAN * z * zzh;
}
__device__ __forceinline__ double cube(double x) { return (x * x) * x; }

__device__ __forceinline__ double rair() { return RGAS * 1.0e3 / XMAIR; }
__device__ __forceinline__ double zcrdq() { return 1.0 / (rair() / 461.51) - 1.0; }

__global__ void k_kzz_rows(KArgs A) {
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= A.jm) return;
    const double GTOR = PI_ / 180.0;
    const double lat = A.ybeg + 0.5 * A.dy + A.dy * j;
    A.dxx[j] = AE * A.dx * GTOR * gbm_cos(lat * GTOR);
}

__global__ void __launch_bounds__(GB_TUNE_MAX_CELL) k_kzz_levels(KArgs A) {
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const int lm = A.lm;
    if (t >= (int64_t)A.im * A.jm * lm) return;
    const int64_t c = t / lm;
    const int l = (int)(t % lm);
    const int i = (int)(c / A.jm), j = (int)(c % A.jm);
    const double ZKAPPA = rair() / CP_AIR, ZCRDQ = zcrdq();
    const double sm = S2(A.spm, i, j);
    const double ph0 = A.at[l] + A.bt[l] * sm, ph1 = A.at[l + 1] + A.bt[l + 1] * sm;
    const double m = div_by_recip((ph0 - ph1) * A.dxyp[j], GRAV, RGRAV);
    const double pf = (ph0 + ph1) * 0.5;
    const double tl = S3(A.t, i, j, l), ql = S3(A.q, i, j, l);
    const double wthm = tl * gbm_pow(div_ip(APZERO, pf), ZKAPPA);
    A.wthm[t] = wthm;
    A.zthvk[t] = wthm * (1.0 + ZCRDQ * ql);
    A.lpf[t] = gbm_log(pf);
    if (l >= 1) A.lphlb[t] = gbm_log(ph0);
    if (l < lm - 1) {  // the geopotential increment of layer l: gph(l+1) = gph(l) + this
        const double s = S2(A.sp, i, j);
        const double tv = tl * (1.0 + 0.608 * ql);
        const double pdown = A.at[l] + A.bt[l] * s, pup = A.at[l + 1] + A.bt[l + 1] * s;
        A.dzg[t] = div_by_recip(tv * 287.05 * gbm_log(div_ip(pdown, pup)), GRAV, RGRAV);
    }
    const double dyy = AE * A.dy * (PI_ / 180.0);
    A.uw[t] = div_ip(A.dxx[j] * (S3(A.pu, i + 1, j, l) + S3(A.pu, i, j, l)) * 0.5, m);
    A.vw[t] = div_ip(dyy * (S3(A.pv, i, j + 1, l) + S3(A.pv, i, j, l)) * 0.5, m);
}

// The bulk-Richardson sweep up a column (diffusion.py:123-152), split where its terms allow:
// each level's Richardson number before the running mask,
//   zrino(k) = GRAV (tkv(k) - ref) dz(k) / (wtseff vvk(k)) + copysign(1e-10, .)
// (first pass: ref = wtseff; second: ref = the parcel's thvparc, the product vvk wtseff), needs
// only the column's constants, so it is computed a thread per (column, level) (k_kzz_heights,
// k_kzz_raw2); the carried part -- the mask jwork, the last Richardson number, pblh -- runs a
// thread per column (sweep_carry).
__device__ double sweep_carry(double pblh, const double *whm, const double *raw, int k0, int lm) {
    // jwork and jq are flags (+0.0 or 1.0): their products and blends are integer selects
    // (mul01, blend01); wrino = zrino + (1 - jwork) 0.1 is zrino + +0 while jwork is 1
    double jwork = 1.0, wrino = 0.0;
    for (int k = k0; k < lm; ++k) {
        const double zrino = mul01(jwork, raw[k]);
        const double jq = jqif_ip(RICR, zrino);
        const double frac = div_ip(RICR - wrino, zrino - wrino);
        const double at_ricr = (k == 0) ? frac * whm[k] : whm[k - 1] + frac * (whm[k] - whm[k - 1]);
        pblh = blend01(jq, pblh, at_ricr);
        jwork = flag(on(jq) && on(jwork));
        wrino = on(jwork) ? blend01(1.0, zrino, 0.1) : zrino + 0.1;  // zrino + (1 - jwork) 0.1
    }
    // (1 - jwork) pblh + whm(lm-1) jwork, or with the second product's factors swapped (the same value)
    return blend01(jwork, whm[lm - 1], pblh);
}

// thread per column: the geopotential's running sum, ustar (diffusion.py:76-89), the surface
// fluxes and the Obukhov length (diffusion.py:155-170) into the column values
__global__ void __launch_bounds__(GB_TUNE_MAX_COLUMN) k_kzz_surface(KArgs A) {
    const int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= (int64_t)A.im * A.jm) return;
    const int i = (int)(c / A.jm), j = (int)(c % A.jm);
    const int lm = A.lm;
    const double ZCRDQ = zcrdq();
    double *gph = A.gph + c * (lm + 1);
    const double *dzg = A.dzg + c * lm, *wthm = A.wthm + c * lm;
    const double sm = S2(A.spm, i, j);

    const double g0 = div_by_recip(S2(A.surf[0], i, j), GRAV, RGRAV);
    gph[0] = g0;
    double g = g0, g1 = g0;
    for (int k = 0; k < lm - 1; ++k) {
        g = g + dzg[k];
        gph[k + 1] = g;
        if (k == 0) g1 = g;
    }
    gph[lm] = 200000.0;

    const double xland = div_by_recip(S2(A.surf[1], i, j), 100.0, 0.01);  // 0.01 = RN(1 / 100)
    const double ew = S2(A.surf[8], i, j), ns = S2(A.surf[9], i, j);
    const double tau = sqrt_ip(ew * ew + ns * ns);
    const double ustar_sea = np_max(0.001, sqrt_ip(div_ip(tau, RHO_AIR)));
    const double u10 = S2(A.surf[4], i, j), v10 = S2(A.surf[5], i, j);
    const double wind10m = sqrt_ip(u10 * u10 + v10 * v10);
    const double sr_land = np_max(1e-2, S2(A.surf[3], i, j));
    const double sr_help = np_min(S2(A.surf[2], i, j), 0.03);
    double land = div_ip(VKARMAN * wind10m, gbm_log(div_ip(10.0, sr_help))) * gbm_log(div_ip(75.0, sr_help));
    land = div_ip(land, gbm_log(div_ip(10.0, sr_land)));
    const double ustar_land = gb_gt0(xland) ? land : 0.0;
    const double ustar_loc = xland * ustar_land + (1.0 - xland) * ustar_sea;

    const double ph0 = A.at[0] + A.bt[0] * sm, ph1 = A.at[1] + A.bt[1] * sm;
    const double dz1 = (lm > 1 ? g1 : gph[1]) - g0, dp1 = ph0 - ph1;
    const double wheat = div_ip(div_ip(-S2(A.surf[6], i, j) * dz1 * GRAV, dp1), CP_AIR);
    const double wqflx = div_ip(div_ip(-S2(A.surf[7], i, j) * dz1 * GRAV, dp1), LVAP);
    const double ustr = np_max(ustar_loc, 0.01);
    const double wtseff = wthm[0] * (1.0 + ZCRDQ * S3(A.q, i, j, 0));
    const double wheatv = wheat + ZCRDQ * wthm[0] * wqflx;
    const double wobkl = div_ip(-wtseff * cube(ustr), GRAV * VKARMAN * (wheatv + copysign(1.0e-10, wheatv)));
    double *cv = A.col + c * NCOLVAL;
    cv[0] = g0;
    cv[2] = wobkl;
    cv[3] = wheatv;
    cv[4] = ustr;
    cv[10] = wtseff;
}

// the height of level l above the surface (mass_t, diffusion.py:107-120)
__device__ __forceinline__ double level_height(const KArgs &A, const double *gph, double z0, double sm, int l) {
    const double ph0 = A.at[l] + A.bt[l] * sm, ph1 = A.at[l + 1] + A.bt[l + 1] * sm;
    const double pf = (ph0 + ph1) * 0.5;
    // about 0.5, at a binade's edge, where div_ip would take the division itself after its own work
    const double intfac = (ph0 - pf) / (ph0 - ph1);
    return (gph[l] - z0) * (1.0 - intfac) + (gph[l + 1] - z0) * intfac;
}

// thread per (column, level): the level height, and the first sweep's level terms
__global__ void __launch_bounds__(GB_TUNE_MAX_CELL) k_kzz_heights(KArgs A) {
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const int lm = A.lm;
    if (t >= (int64_t)A.im * A.jm * lm) return;
    const int64_t c = t / lm;
    const int k = (int)(t % lm);
    const int i = (int)(c / A.jm), j = (int)(c % A.jm);
    const double *gph = A.gph + c * (lm + 1), *cv = A.col + c * NCOLVAL;
    const double z0 = cv[0], ustr = cv[4], wtseff = cv[10];
    const double sm = S2(A.spm, i, j);
    const double whk = level_height(A, gph, z0, sm, k), wh0 = level_height(A, gph, z0, sm, 0);
    A.whm[t] = whk;
    const double *uw = A.uw + c * lm, *vw = A.vw + c * lm;
    const double du = uw[k] - uw[0], dv = vw[k] - vw[0];
    const double vvk = np_max(du * du + dv * dv + ZACB * ustr * ustr, TINY);
    const double dz = whk - wh0;
    double zrino = div_ip(GRAV * (A.zthvk[t] - wtseff) * dz, wtseff * vvk);
    zrino = add_ip(zrino, copysign(1.0e-10, zrino));  // like-signed: the integer pipe's sum
    A.sw_vvk[t] = vvk;
    A.sw_dz[t] = dz;
    A.sw_raw[t] = zrino;
}

// thread per column: the first sweep (pblh from 0), the parcel's excess (diffusion.py:171-178)
__global__ void __launch_bounds__(GB_TUNE_MAX_COLUMN) k_kzz_sweep1(KArgs A) {
    const int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= (int64_t)A.im * A.jm) return;
    const int lm = A.lm;
    const double ONET = 1.0 / 3.0, BINM = 15.0 * SFFRAC;
    double *cv = A.col + c * NCOLVAL;
    const double wobkl = cv[2], wheatv = cv[3], ustr = cv[4], wtseff = cv[10];
    const double pblh = sweep_carry(0.0, A.whm + c * lm, A.sw_raw + c * lm, 0, lm);
    const double jq = jqif(wheatv, 0.0);
    const double fmt = gbm_pow(blend01(jq, 1.0 - div_ip(BINM * pblh, wobkl), 1.0), ONET);
    const double wsc = ustr * fmt;
    const double zexcess = div_ip(wheatv * FAK, wsc);
    cv[1] = pblh;
    cv[11] = wtseff + mul01(jq, zexcess);  // thvparc
}

// thread per (column, level >= 1): the second sweep's level terms
__global__ void __launch_bounds__(GB_TUNE_MAX_CELL) k_kzz_raw2(KArgs A) {
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const int lm = A.lm;
    if (t >= (int64_t)A.im * A.jm * lm) return;
    const int64_t c = t / lm;
    if (t % lm == 0) return;
    const double *cv = A.col + c * NCOLVAL;
    const double wtseff = cv[10], thvparc = cv[11];
    double zrino = div_ip(GRAV * (A.zthvk[t] - thvparc) * A.sw_dz[t], A.sw_vvk[t] * wtseff);
    zrino = add_ip(zrino, copysign(1.0e-10, zrino));  // like-signed: the integer pipe's sum
    A.sw_raw[t] = zrino;
}

// thread per column: the second sweep, pblh, and the interfaces' column constants: w* and the
// Prandtl term's stability for jq3 = 0 (obukov = 0 * wobkl - 1) and jq3 = 1 (obukov = 1 * wobkl - 0)
__global__ void __launch_bounds__(GB_TUNE_MAX_COLUMN) k_kzz_sweep2(KArgs A) {
    const int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= (int64_t)A.im * A.jm) return;
    const int i = (int)(c / A.jm), j = (int)(c % A.jm);
    const int lm = A.lm;
    const double ONET = 1.0 / 3.0;
    double *cv = A.col + c * NCOLVAL;
    const double wobkl = cv[2], wheatv = cv[3], wtseff = cv[10];
    double pblh = sweep_carry(cv[1], A.whm + c * lm, A.sw_raw + c * lm, 1, lm);
    pblh = np_max(pblh, 100.0);
    if (A.pblh.p) A.pblh.p[(int64_t)i * A.pblh.s0 + (int64_t)j * A.pblh.s1] = pblh;
    cv[1] = pblh;
    cv[5] = gbm_pow(fabs(wheatv) * GRAV * pblh / wtseff, ONET);
    const double stab0 = 1.0 - SSFRAC * BETAH * pblh / (0.0 * wobkl - 1.0);
    const double stab1 = 1.0 - SSFRAC * BETAH * pblh / (1.0 * wobkl - 0.0);
    cv[6] = gbm_pow(stab0, ONET);
    cv[7] = sqrt_ip(stab0);
    cv[8] = gbm_pow(stab1, ONET);
    cv[9] = sqrt_ip(stab1);
    // the interface's pr = jq3 (t1 / t2 + CCON FAKN w* / (U t1)) + (1 - jq3) takes t1, t2 from one of
    // the two pairs above: both sums, each in the statement's own order
    const double CCON = SFFRAC * VKARMAN, zwstr = cv[5], U = cv[4];
    cv[12] = cv[6] / cv[7] + CCON * FAKN * zwstr / (U * cv[6]);
    cv[13] = cv[8] / cv[9] + CCON * FAKN * zwstr / (U * cv[8]);
    cv[14] = recip_for(cv[13]);
    const double stabw = 1.0 - SSFRAC * BETAH * pblh / wobkl;
    cv[15] = stabw;
    cv[16] = gbm_pow(stabw, ONET);
    cv[17] = recip_for(pblh);
    cv[18] = recip_for(wobkl);
}

// Lanes run along the columns and warps along the interfaces (a block: 32 columns at blockDim / 32
// consecutive interfaces): the boundary layer's branches (the powers of its stability terms,
// pow(1, y) = 1 returning at once above it) are then taken or left by whole warps.
__global__ void __launch_bounds__(GB_TUNE_MAX_CELL) k_kzz_interfaces(KArgs A) {
    const int lm = A.lm, ni = lm - 1, lv = blockDim.x >> 5;
    const int nkg = (ni + lv - 1) / lv;
    const int64_t c = (int64_t)(blockIdx.x / nkg) * 32 + (threadIdx.x & 31);
    const int k = (int)(blockIdx.x % nkg) * lv + (int)(threadIdx.x >> 5) + 1;  // interface k, between layers k-1 and k
    if (c >= (int64_t)A.im * A.jm || k > ni) return;
    const int i = (int)(c / A.jm), j = (int)(c % A.jm);
    const double ONET = 1.0 / 3.0;
    const double *cv = A.col + c * NCOLVAL;
    const double z0 = cv[0], P = cv[1], Wb = cv[2], HV = cv[3], U = cv[4];
    const double yP = cv[17], yWb = cv[18];
    const int64_t ck = c * lm + k;
    const double *gph = A.gph + c * (lm + 1);

    const double z = gph[k] - z0;
    double jq = jqif(1000.0, z);
    const double zlambdac = blend01(jq, 300.0, 30.0 + 270.0 * gbm_exp(1.0 - div_by_recip(z, 1000.0, 1.0e-3)));
    const double rkz = div_ip(1.0, VKARMAN * z);
    double cml2 = div_ip(1.0, div_ip(1.0, zlambdac) + rkz);
    cml2 = cml2 * cml2;
    const double du = A.uw[ck] - A.uw[ck - 1], dv = A.vw[ck] - A.vw[ck - 1];
    double zdup2 = np_max(du * du + dv * dv, 1.0e-10);
    const double whk = A.whm[ck], whk1 = A.whm[ck - 1];
    const double zdz = whk - whk1;
    zdup2 = div_ip(zdup2, zdz * zdz);
    const double arg = div_ip(A.lphlb[ck] - A.lpf[ck - 1], A.lpf[ck] - A.lpf[ck - 1]);
    const double dthv = A.zthvk[ck] - A.zthvk[ck - 1];
    const double zthva = A.zthvk[ck - 1] + arg * dthv;
    const double zsstab = div_ip(div_ip(GRAV, zthva) * dthv, zdz);
    const double zrinub = div_ip(zsstab, zdup2);
    const double zfunst = sqrt_ip(np_max(1.0 - 18.0 * zrinub, 0.0));
    double zfstabh = div_ip(1.0, 1.0 + 10.0 * zrinub * (1.0 + 8.0 * zrinub));
    const double rdup = sqrt_ip(zdup2);
    const double zkvn = cml2 * rdup;
    jq = jqif(zrinub, 0.0);
    const double wkvf = blend01(jq, np_max(CKMIN, zkvn * zfstabh), np_max(CKMIN, zkvn * zfunst));
    jq = jqif(P, z);
    const double jz = mul01(jq, z);
    const double zh = div_by_recip(jz, P, yP);
    const double zl = div_by_recip(jz, Wb, yWb) + (1.0 - jq);
    const double zzh = mul01(jq, (1.0 - zh) * (1.0 - zh));
    double jq1 = jqif(HV, 0.0);
    const double jq2 = flag(on(jq) && !on(jq1)), jq3 = flag(on(jq) && on(jq1));
    const double jq6 = flag(on(jq1) && on(jqif(P, whk1)) && on(jqif(whk, P)));
    jq1 = jqif(SFFRAC, zh);
    const double jq4 = flag(on(jq3) && on(jq1)), jq5 = flag(on(jq3) && !on(jq1));
    cml2 = div_ip(1.0, rkz + 1.0 / 450.0);
    cml2 = cml2 * cml2;
    const double jqq = jqif(zrinub, 0.0);
    zfstabh = div_ip(jqq, 1.0 + 10.0 * zrinub * sqrt_ip(1.0 + mul01(jqq, zrinub))) + (1.0 - jqq);
    double zpblk = cml2 * rdup * zfstabh;
    const double zkvh = blend01(jq2, np_max(zpblk, KVHMIN), wkvf);
    double zslask = 1.0 - BETAH * zl;
    zslask = blend01(jq4, zslask, 1.0);
    zpblk = blend01(jq4, U * VKARMAN * z * zzh * gbm_pow(zslask, ONET), zkvh);  // (1 - jq4) zkvh + jq4 (...)
    // jq5 is 0 or 1: at 1 the base is the column's stabw (stabw + 0.0, whose cube root is stabw's)
    const bool jq5_on = (__double_as_longlong(jq5) << 1) != 0;
    double fmt;
    if (jq5_on) {
        fmt = cv[16];
    } else {
        zslask = blend01(jq5, cv[15], 1.0);
        fmt = gbm_pow(zslask, ONET);
    }
    const double wsc = U * fmt;
    // (1 - jq5) zpblk + (((jq5 wsc) VKARMAN) z) zzh: at jq5 = 1 the product (1 wsc = wsc) plus +0
    // zpblk; at jq5 = 0 zpblk plus a zero of the sign of wsc z zzh (a NaN if any is not finite)
    {
        const unsigned long long bw = (unsigned long long)__double_as_longlong(wsc), bz = (unsigned long long)__double_as_longlong(z),
                                 bh = (unsigned long long)__double_as_longlong(zzh), bp = (unsigned long long)__double_as_longlong(zpblk);
        if (jq5_on) {
            zpblk = blend01(1.0, wsc * VKARMAN * z * zzh, zpblk);
        } else if (finite_bits(bw) && finite_bits(bz) && finite_bits(bh) && finite_bits(bp)) {
            const unsigned long long zs = (bw ^ bz ^ bh) & 0x8000000000000000ULL;  // the zero's sign
            if (bp == 0x8000000000000000ULL && zs == 0) zpblk = 0.0;               // -0 + +0 = +0
        } else {
            zpblk = zpblk_jq5_fp64(jq5, zpblk, wsc, z, zzh);
        }
    }
    const bool jq3_on = (__double_as_longlong(jq3) << 1) != 0;  // jq3 != 0.0, on the integer pipe
    const double pr = blend01(jq3, jq3_on ? cv[13] : cv[12], 1.0);
    // pr's reciprocal: the sum's at jq3 = 1 (pr = sum + 0.0), 1 where jq3 = 0 left pr at exactly 1,
    // else none (div_by_recip divides)
    const double ypr = jq3_on ? cv[14] : (__double_as_longlong(pr) == 0x3ff0000000000000LL ? 1.0 : 0.0);
    const double kv = blend01(jq3, np_max(div_by_recip(zpblk, pr, ypr), KVHMIN), zkvh);
    const double thvgrad = div_ip(dthv, zdz);
    const double kvhentr = div_ip(0.2 * HV, thvgrad);
    const double kvh = blend01(jq6, kvhentr, kv);

    // dkg across interface l + 1 = k for l < lmax - 1, zero at lmax - 1 (diffusion.py:256-263)
    const int l = k - 1;
    if (l < A.lmax - 1) {
        const double sm = S2(A.spm, i, j);
        const double p0 = A.at[l] + A.bt[l] * sm, p1 = A.at[l + 1] + A.bt[l + 1] * sm,
                     p2 = A.at[l + 2] + A.bt[l + 2] * sm;
        const double m0 = div_by_recip((p0 - p1) * A.dxyp[j], GRAV, RGRAV),
                     m1 = div_by_recip((p1 - p2) * A.dxyp[j], GRAV, RGRAV);
        const double dz = gph[l + 2] - gph[l];
        S3(A.dkg, i, j, l) = div_ip(np_max(0.0, kvh) * 2.0 * (m1 + m0), dz * dz);
    }
    if (k == 1) S3(A.dkg, i, j, A.lmax - 1) = 0.0;
}

}  // namespace

extern "C" int gb_calc_kzz(gb_ctx *ctx, const gb_view *spm, const gb_view *sp, const gb_view *pu, const gb_view *pv,
                           const gb_view *t, const gb_view *q, const gb_view *surface, const double *at,
                           const double *bt, const double *dxyp, int lmax_conv, double dx, double dy, double ybeg,
                           const gb_view *dkg, const gb_view *pblh) {
    if (!ctx || !spm || !sp || !pu || !pv || !t || !q || !surface || !at || !bt || !dxyp || !dkg) return GB_EARG;
    KArgs A{};
    A.spm = dv(spm); A.sp = dv(sp); A.pu = dv(pu); A.pv = dv(pv); A.t = dv(t); A.q = dv(q);
    for (int k = 0; k < 10; ++k) A.surf[k] = dv(&surface[k]);
    A.dkg = dv(dkg);
    A.pblh = pblh ? dv(pblh) : DV{};
    A.at = at; A.bt = bt; A.dxyp = dxyp;
    A.im = (int)t->n[0]; A.jm = (int)t->n[1]; A.lm = (int)t->n[2]; A.lmax = lmax_conv;
    A.dx = dx; A.dy = dy; A.ybeg = ybeg;
    if (lmax_conv < 1 || lmax_conv > A.lm || A.lm < 2) {
        gb_set_error("gb_calc_kzz: need 1 <= lmax_conv <= lm and lm >= 2");
        return GB_EARG;
    }
    const int64_t ncol = (int64_t)A.im * A.jm, ncell = ncol * A.lm;
    const size_t doubles = (size_t)A.jm + 11 * (size_t)ncell + (size_t)ncol * (A.lm + 1) + (size_t)ncol * NCOLVAL;
    double *w = gb_work(ctx, doubles * sizeof(double));
    if (!w) return GB_ECUDA;
    A.dxx = w; w += A.jm;
    A.wthm = w; w += ncell;
    A.zthvk = w; w += ncell;
    A.lpf = w; w += ncell;
    A.lphlb = w; w += ncell;
    A.dzg = w; w += ncell;
    A.uw = w; w += ncell;
    A.vw = w; w += ncell;
    A.whm = w; w += ncell;
    A.sw_vvk = w; w += ncell;
    A.sw_dz = w; w += ncell;
    A.sw_raw = w; w += ncell;
    A.gph = w; w += ncol * (A.lm + 1);
    A.col = w;
    const int tcol = ctx->tune[GB_TUNE_COLUMN_THREADS], tcell = ctx->tune[GB_TUNE_CELL_THREADS];
    k_kzz_rows<<<gb_blocks(A.jm, 128), 128, 0, ctx->stream>>>(A);
    if (int rc = gb_after_launch(ctx, "kzz_rows")) return rc;
    k_kzz_levels<<<gb_blocks(ncell, tcell), tcell, 0, ctx->stream>>>(A);
    if (int rc = gb_after_launch(ctx, "kzz_levels")) return rc;
    k_kzz_surface<<<gb_blocks(ncol, tcol), tcol, 0, ctx->stream>>>(A);
    if (int rc = gb_after_launch(ctx, "kzz_surface")) return rc;
    k_kzz_heights<<<gb_blocks(ncell, tcell), tcell, 0, ctx->stream>>>(A);
    if (int rc = gb_after_launch(ctx, "kzz_heights")) return rc;
    k_kzz_sweep1<<<gb_blocks(ncol, tcol), tcol, 0, ctx->stream>>>(A);
    if (int rc = gb_after_launch(ctx, "kzz_sweep1")) return rc;
    k_kzz_raw2<<<gb_blocks(ncell, tcell), tcell, 0, ctx->stream>>>(A);
    if (int rc = gb_after_launch(ctx, "kzz_raw2")) return rc;
    k_kzz_sweep2<<<gb_blocks(ncol, tcol), tcol, 0, ctx->stream>>>(A);
    if (int rc = gb_after_launch(ctx, "kzz_sweep2")) return rc;
    // blocks of 32 columns x (tcell / 32) interfaces
    const int lv = tcell / 32;
    k_kzz_interfaces<<<(unsigned)((ncol + 31) / 32 * ((A.lm - 1 + lv - 1) / lv)), tcell, 0, ctx->stream>>>(A);
    return gb_after_launch(ctx, "kzz_interfaces");
}
