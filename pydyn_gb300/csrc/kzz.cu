// Calc_Kzz: the vertical diffusion exchange rate dkg of every column of a region, one warp per
// column.  Lanes take the levels for the level-parallel work (the potential temperatures,
// logarithms, winds, the Richardson-number diffusivities), lane 0 the two sequential
// boundary-layer-height sweeps and the geopotential's running sum; the powers that depend on the
// column alone (w* and the Prandtl stability term) are computed once and shared.  Every value is
// the per-element statement of the reference in its order; exp / log / pow / cos are gbmath.h.
// Reference: pydyn diffusion.py:71-276 (jqif, ustar, geopotential, mass_t, _winds, _pbl_pass,
// bldiff, dkg, calc_kzz).
#include "gb_common.cuh"
#include "gbmath.h"

namespace {

constexpr int WARPS = 8;

struct KArgs {
    DV spm, sp, pu, pv, t, q, surf[10], dkg, pblh;
    const double *at, *bt, *dxyp;
    int im, jm, lm, lmax;
    double dx, dy, ybeg;
};

constexpr double GRAV = 9.80665, PI_ = 3.14159265358979, AE = 6.371e6, VKARMAN = 0.4, CP_AIR = 1004.0;
constexpr double LVAP = 2.5e6, RGAS = 8.3144, XMAIR = 28.94, RHO_AIR = 1.2, CKMIN = 1.0e-15, SFFRAC = 0.1;
constexpr double APZERO = 100000.0, BETAH = 15.0, FAK = 8.5, FAKN = 7.2, TINY = 1.0e-9, ZACB = 100.0;
constexpr double RICR = 0.3, SSFRAC = 0.1, KVHMIN = 0.1;

__device__ __forceinline__ double S2(const DV &v, int i, int j) { return v.p[(int64_t)i * v.s0 + (int64_t)j * v.s1]; }
__device__ __forceinline__ double &S3(const DV &v, int i, int j, int l) {
    return v.p[(int64_t)i * v.s0 + (int64_t)j * v.s1 + (int64_t)l * v.s2];
}
// jqif(x, y) = nint(0.5 + sign(0.5, x - y)): 1 where x - y has a clear sign bit
__device__ __forceinline__ double jqif(double x, double y) { return signbit(x - y) ? 0.0 : 1.0; }
__device__ __forceinline__ double cube(double x) { return (x * x) * x; }

// one sweep of the bulk Richardson number up the column (diffusion.py:123-152)
__device__ double pbl_sweep(double pblh, const double *whm, const double *uw, const double *vw, const double *wthm,
                            const double *qc, double ustr, double wtseff, double ref, bool first, int lm,
                            double zcrdq) {
    double jwork = 1.0, wrino = 0.0;
    for (int k = first ? 0 : 1; k < lm; ++k) {
        const double du = uw[k] - uw[0], dv = vw[k] - vw[0];
        const double vvk = np_max(du * du + dv * dv + ZACB * ustr * ustr, TINY);
        const double tkv = wthm[k] * (1.0 + zcrdq * qc[k]);
        const double dz = whm[k] - whm[0];
        double zrino = first ? GRAV * (tkv - wtseff) * dz / (wtseff * vvk) : GRAV * (tkv - ref) * dz / (vvk * wtseff);
        zrino = zrino + copysign(1.0e-10, zrino);
        zrino = jwork * zrino;
        const double jq = jqif(RICR, zrino);
        const double frac = (RICR - wrino) / (zrino - wrino);
        const double at_ricr = (k == 0) ? frac * whm[k] : whm[k - 1] + frac * (whm[k] - whm[k - 1]);
        pblh = jq * pblh + (1.0 - jq) * at_ricr;
        jwork = jq * jwork;
        wrino = zrino + (1.0 - jwork) * 0.1;
    }
    return first ? (1.0 - jwork) * pblh + whm[lm - 1] * jwork : (1.0 - jwork) * pblh + jwork * whm[lm - 1];
}

__global__ void __launch_bounds__(WARPS * 32) k_calc_kzz(KArgs A) {
    extern __shared__ double smem[];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int64_t col = (int64_t)blockIdx.x * WARPS + warp;
    if (col >= (int64_t)A.im * A.jm) return;
    const int i = (int)(col / A.jm), j = (int)(col % A.jm);
    const int lm = A.lm, W = lm + 2;
    double *gph = smem + (size_t)warp * 12 * W;
    double *phlb = gph + W, *m = phlb + W, *pf = m + W, *wthm = pf + W, *zthvk = wthm + W, *whm = zthvk + W;
    double *uw = whm + W, *vw = uw + W, *qc = vw + W, *kvh = qc + W, *lpf = kvh + W;

    const double RAIR = RGAS * 1.0e3 / XMAIR, EPSILO = RAIR / 461.51, ZKAPPA = RAIR / CP_AIR;
    const double ZCRDQ = 1.0 / EPSILO - 1.0, ONET = 1.0 / 3.0, CCON = SFFRAC * VKARMAN, BINM = 15.0 * SFFRAC;
    const double GTOR = PI_ / 180.0;
    const double lat = A.ybeg + 0.5 * A.dy + A.dy * j;
    const double dxx = AE * A.dx * GTOR * gbm_cos(lat * GTOR), dyy = AE * A.dy * GTOR;
    const double s = S2(A.sp, i, j), sm = S2(A.spm, i, j);

    // ---- per level: phlb, m, pf, theta, the log-pressure increments of the geopotential
    for (int l = lane; l <= lm; l += 32) phlb[l] = A.at[l] + A.bt[l] * sm;
    __syncwarp();
    for (int l = lane; l < lm; l += 32) {
        const double tl = S3(A.t, i, j, l), ql = S3(A.q, i, j, l);
        qc[l] = ql;
        m[l] = (phlb[l] - phlb[l + 1]) * A.dxyp[j] / GRAV;
        pf[l] = (phlb[l] + phlb[l + 1]) * 0.5;
        wthm[l] = tl * gbm_pow(APZERO / pf[l], ZKAPPA);
        zthvk[l] = wthm[l] * (1.0 + ZCRDQ * ql);
        lpf[l] = gbm_log(pf[l]);
        if (l < lm - 1) {  // gph increment of layer l (gph(l+1) = gph(l) + this)
            const double tv = tl * (1.0 + 0.608 * ql);
            const double pdown = A.at[l] + A.bt[l] * s, pup = A.at[l + 1] + A.bt[l + 1] * s;
            kvh[l] = tv * 287.05 * gbm_log(pdown / pup) / GRAV;  // kvh as scratch for now
        }
        uw[l] = dxx * (S3(A.pu, i + 1, j, l) + S3(A.pu, i, j, l)) * 0.5 / m[l];
        vw[l] = dyy * (S3(A.pv, i, j + 1, l) + S3(A.pv, i, j, l)) * 0.5 / m[l];
    }
    __syncwarp();
    if (lane == 0) {  // the geopotential's running sum up the column
        gph[0] = S2(A.surf[0], i, j) / GRAV;
        for (int k = 0; k < lm - 1; ++k) gph[k + 1] = gph[k] + kvh[k];
        gph[lm] = 200000.0;
    }
    __syncwarp();
    const double z0 = gph[0];
    for (int l = lane; l < lm; l += 32) {
        const double intfac = (phlb[l] - pf[l]) / (phlb[l] - phlb[l + 1]);
        whm[l] = (gph[l] - z0) * (1.0 - intfac) + (gph[l + 1] - z0) * intfac;
    }
    __syncwarp();

    // ---- the column's surface quantities and its boundary-layer height (lane 0, broadcast)
    double P = 0.0, Wb = 0.0, HV = 0.0, U = 0.0, TS = 0.0, zwstr = 0.0, t1a = 0.0, t2a = 0.0, t1b = 0.0, t2b = 0.0;
    if (lane == 0) {
        const double xland = S2(A.surf[1], i, j) / 100.0;
        const double ew = S2(A.surf[8], i, j), ns = S2(A.surf[9], i, j);
        const double tau = sqrt(ew * ew + ns * ns);
        const double ustar_sea = np_max(0.001, sqrt(tau / RHO_AIR));
        const double u10 = S2(A.surf[4], i, j), v10 = S2(A.surf[5], i, j);
        const double wind10m = sqrt(u10 * u10 + v10 * v10);
        const double sr_land = np_max(1e-2, S2(A.surf[3], i, j));
        const double sr_help = np_min(S2(A.surf[2], i, j), 0.03);
        double land = VKARMAN * wind10m / gbm_log(10.0 / sr_help) * gbm_log(75.0 / sr_help);
        land = land / gbm_log(10.0 / sr_land);
        const double ustar_land = xland > 0.0 ? land : 0.0;
        const double ustar_loc = xland * ustar_land + (1.0 - xland) * ustar_sea;
        const double dz1 = gph[1] - gph[0], dp1 = phlb[0] - phlb[1];
        const double wheat = -S2(A.surf[6], i, j) * dz1 * GRAV / dp1 / CP_AIR;
        const double wqflx = -S2(A.surf[7], i, j) * dz1 * GRAV / dp1 / LVAP;
        const double ustr = np_max(ustar_loc, 0.01);
        const double wtseff = wthm[0] * (1.0 + ZCRDQ * qc[0]);
        const double wheatv = wheat + ZCRDQ * wthm[0] * wqflx;
        const double wobkl = -wtseff * cube(ustr) / (GRAV * VKARMAN * (wheatv + copysign(1.0e-10, wheatv)));
        double pblh = pbl_sweep(0.0, whm, uw, vw, wthm, qc, ustr, wtseff, 0.0, true, lm, ZCRDQ);
        const double jq = jqif(wheatv, 0.0);
        const double fmt = gbm_pow(jq * (1.0 - BINM * pblh / wobkl) + (1.0 - jq), ONET);
        const double wsc = ustr * fmt;
        const double zexcess = wheatv * FAK / wsc;
        const double thvparc = wtseff + jq * zexcess;
        pblh = pbl_sweep(pblh, whm, uw, vw, wthm, qc, ustr, wtseff, thvparc, false, lm, ZCRDQ);
        pblh = np_max(pblh, 100.0);
        P = pblh; Wb = wobkl; HV = wheatv; U = ustr; TS = wtseff;
        zwstr = gbm_pow(fabs(HV) * GRAV * P / TS, ONET);  // the same at every interface
        // the Prandtl term's stability for jq3 = 0 (obukov = -1) and jq3 = 1 (obukov = wobkl)
        const double stab0 = 1.0 - SSFRAC * BETAH * P / (0.0 * Wb - 1.0);
        const double stab1 = 1.0 - SSFRAC * BETAH * P / (1.0 * Wb - 0.0);
        t1a = gbm_pow(stab0, ONET); t2a = sqrt(stab0);
        t1b = gbm_pow(stab1, ONET); t2b = sqrt(stab1);
        if (A.pblh.p) A.pblh.p[(int64_t)i * A.pblh.s0 + (int64_t)j * A.pblh.s1] = pblh;
    }
    P = __shfl_sync(FULL_MASK, P, 0);
    Wb = __shfl_sync(FULL_MASK, Wb, 0);
    HV = __shfl_sync(FULL_MASK, HV, 0);
    U = __shfl_sync(FULL_MASK, U, 0);
    TS = __shfl_sync(FULL_MASK, TS, 0);
    zwstr = __shfl_sync(FULL_MASK, zwstr, 0);
    t1a = __shfl_sync(FULL_MASK, t1a, 0);
    t2a = __shfl_sync(FULL_MASK, t2a, 0);
    t1b = __shfl_sync(FULL_MASK, t1b, 0);
    t2b = __shfl_sync(FULL_MASK, t2b, 0);

    // ---- the diffusivity at every interface k (between layers k-1 and k), lanes across k
    for (int k = 1 + lane; k < lm; k += 32) {
        const double z = gph[k] - z0;
        double jq = jqif(1000.0, z);
        const double zlambdac = jq * 300.0 + (1.0 - jq) * (30.0 + 270.0 * gbm_exp(1.0 - z / 1000.0));
        double cml2 = 1.0 / (1.0 / zlambdac + 1.0 / (VKARMAN * z));
        cml2 = cml2 * cml2;
        const double du = uw[k] - uw[k - 1], dv = vw[k] - vw[k - 1];
        double zdup2 = np_max(du * du + dv * dv, 1.0e-10);
        const double zdz = whm[k] - whm[k - 1];
        zdup2 = zdup2 / (zdz * zdz);
        const double arg = (gbm_log(phlb[k]) - lpf[k - 1]) / (lpf[k] - lpf[k - 1]);
        const double dthv = zthvk[k] - zthvk[k - 1];
        const double zthva = zthvk[k - 1] + arg * dthv;
        const double zsstab = GRAV / zthva * dthv / zdz;
        const double zrinub = zsstab / zdup2;
        const double zfunst = sqrt(np_max(1.0 - 18.0 * zrinub, 0.0));
        double zfstabh = 1.0 / (1.0 + 10.0 * zrinub * (1.0 + 8.0 * zrinub));
        const double zkvn = cml2 * sqrt(zdup2);
        jq = jqif(zrinub, 0.0);
        const double wkvf = jq * np_max(CKMIN, zkvn * zfstabh) + (1.0 - jq) * np_max(CKMIN, zkvn * zfunst);
        jq = jqif(P, z);
        const double zh = jq * z / P;
        const double zl = jq * z / Wb + (1.0 - jq);
        const double zzh = jq * ((1.0 - zh) * (1.0 - zh));
        double jq1 = jqif(HV, 0.0);
        const double jq2 = jq * (1.0 - jq1), jq3 = jq * jq1;
        const double jq6 = jq1 * jqif(P, whm[k - 1]) * jqif(whm[k], P);
        jq1 = jqif(SFFRAC, zh);
        const double jq4 = jq3 * jq1, jq5 = jq3 * (1.0 - jq1);
        cml2 = 1.0 / (1.0 / (VKARMAN * z) + 1.0 / 450.0);
        cml2 = cml2 * cml2;
        const double jqq = jqif(zrinub, 0.0);
        zfstabh = jqq / (1.0 + 10.0 * zrinub * sqrt(1.0 + jqq * zrinub)) + (1.0 - jqq);
        double zpblk = cml2 * sqrt(zdup2) * zfstabh;
        const double zkvh = jq2 * np_max(zpblk, KVHMIN) + (1.0 - jq2) * wkvf;
        double zslask = 1.0 - BETAH * zl;
        zslask = jq4 * zslask + (1.0 - jq4);
        zpblk = (1.0 - jq4) * zkvh + jq4 * (U * VKARMAN * z * zzh * gbm_pow(zslask, ONET));
        zslask = 1.0 - SSFRAC * BETAH * P / Wb;
        zslask = jq5 * zslask + (1.0 - jq5);
        const double fmt = gbm_pow(zslask, ONET);
        const double wsc = U * fmt;
        zpblk = (1.0 - jq5) * zpblk + jq5 * wsc * VKARMAN * z * zzh;
        const double term1 = jq3 != 0.0 ? t1b : t1a, term2 = jq3 != 0.0 ? t2b : t2a;
        const double term3 = CCON * FAKN * zwstr / (U * term1);
        const double pr = jq3 * (term1 / term2 + term3) + (1.0 - jq3);
        const double kv = jq3 * np_max(zpblk / pr, KVHMIN) + (1.0 - jq3) * zkvh;
        const double thvgrad = dthv / zdz;
        const double kvhentr = 0.2 * HV / thvgrad;
        kvh[k - 1] = jq6 * kvhentr + (1.0 - jq6) * kv;
    }
    __syncwarp();
    // ---- dkg across the interfaces l+1, l < lmax-1; zero at lmax-1 (diffusion.py:256-263)
    for (int l = lane; l < A.lmax; l += 32) {
        double v = 0.0;
        if (l < A.lmax - 1) {
            const double dz = gph[l + 2] - gph[l];
            v = np_max(0.0, kvh[l]) * 2.0 * (m[l + 1] + m[l]) / (dz * dz);
        }
        S3(A.dkg, i, j, l) = v;
    }
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
    const size_t smem = (size_t)WARPS * 12 * (A.lm + 2) * sizeof(double);
    GB_CHECK_CUDA(cudaFuncSetAttribute(k_calc_kzz, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    const int64_t cols = (int64_t)A.im * A.jm;
    k_calc_kzz<<<(int)((cols + WARPS - 1) / WARPS), WARPS * 32, smem, ctx->stream>>>(A);
    return gb_after_launch(ctx, "calc_kzz");
}
