/*
 * gbmath.h -- exp, log, pow, sin and cos in IEEE float64 for the host and the device alike.
 *
 * The method is Sun Microsystems' fdlibm 5.3 (freely distributable, published algorithms):
 * exp by reduction x = k ln2 + r and a rational approximation of r; log by reduction to
 * [sqrt(2)/2, sqrt(2)) and a polynomial in s = f / (2 + f); pow by an extra-precise log2(x)
 * (t1 + t2), the product with y split hi / lo, and exp2 of the result; sin / cos by
 * Cody-Waite reduction by pi/2 and minimax kernels.  Special values follow C99 (pow(1, y) = 1).
 * Written for this library from the published method; the same source is compiled for the
 * device (nvcc) and for the host (gcc, -ffp-contract=off), so the results agree bit for bit,
 * and they are within 1 ulp of the C library (tested against glibc).
 */
#ifndef GBMATH_H
#define GBMATH_H

#include <stdint.h>

#if defined(__CUDACC__)
#define GBM_HD __host__ __device__ __forceinline__
#else
#define GBM_HD static inline
#endif

/* The quotients of the main paths.  On the device, div_ip of the kernels' common header (which a
 * device translation unit includes before this file): the correctly rounded quotient, the same
 * bits as a / b, with three FP64 instructions where the FP64 pipe's division issues eight. */
#if defined(__CUDA_ARCH__)
#define GBM_DIV(a, b) div_ip((a), (b))
#else
#define GBM_DIV(a, b) ((a) / (b))
#endif

GBM_HD uint64_t gbm_bits(double x) {
#if defined(__CUDA_ARCH__)
    return (uint64_t)__double_as_longlong(x);
#else
    union { double d; uint64_t u; } c;
    c.d = x;
    return c.u;
#endif
}
GBM_HD double gbm_from(uint64_t u) {
#if defined(__CUDA_ARCH__)
    return __longlong_as_double((long long)u);
#else
    union { double d; uint64_t u; } c;
    c.u = u;
    return c.d;
#endif
}
GBM_HD int32_t gbm_hi(double x) { return (int32_t)(gbm_bits(x) >> 32); }
GBM_HD uint32_t gbm_lo(double x) { return (uint32_t)(gbm_bits(x) & 0xffffffffu); }
GBM_HD double gbm_make(int32_t hi, uint32_t lo) { return gbm_from(((uint64_t)(uint32_t)hi << 32) | lo); }
GBM_HD double gbm_set_hi(double x, int32_t hi) { return gbm_make(hi, gbm_lo(x)); }
GBM_HD double gbm_set_lo(double x, uint32_t lo) { return gbm_make(gbm_hi(x), lo); }
GBM_HD double gbm_fabs(double x) { return gbm_from(gbm_bits(x) & 0x7fffffffffffffffull); }

/* x * 2**n for the n the kernels need (exact unless the result is subnormal: one rounding) */
GBM_HD double gbm_scale2(double x, int n) {
    while (n > 1023) {
        x = x * gbm_make(0x7fe00000, 0);  /* 2**1023 */
        n -= 1023;
    }
    while (n < -1022) {
        if (n >= -1074) return x * gbm_from((uint64_t)1 << (n + 1074));  /* a subnormal power of 2 */
        x = x * gbm_make(0x00100000, 0);  /* 2**-1022 */
        n += 1022;
    }
    return x * gbm_make((int32_t)(n + 1023) << 20, 0);
}

/* ------------------------------------------------------------------ exp */
GBM_HD double gbm_exp(double x) {
    const double one = 1.0, huge = 1.0e+300, twom1000 = 9.33263618503218878990e-302;
    const double o_threshold = 7.09782712893383973096e+02, u_threshold = -7.45133219101941108420e+02;
    const double ln2hi = 6.93147180369123816490e-01, ln2lo = 1.90821492927058770002e-10;
    const double invln2 = 1.44269504088896338700e+00;
    const double P1 = 1.66666666666666019037e-01, P2 = -2.77777777770155933842e-03,
                 P3 = 6.61375632143793436117e-05, P4 = -1.65339022054652515390e-06,
                 P5 = 4.13813679705723846039e-08;
    double y, hi = 0.0, lo = 0.0, c, t;
    int32_t k = 0;
    uint32_t hx = (uint32_t)gbm_hi(x);
    const int xsb = (hx >> 31) & 1;
    hx &= 0x7fffffffu;
    if (hx >= 0x40862E42u) {  /* |x| >= 709.78... */
        if (hx >= 0x7ff00000u) {
            if (((hx & 0xfffffu) | gbm_lo(x)) != 0) return x + x;  /* NaN */
            return xsb == 0 ? x : 0.0;                            /* exp(+-inf) = {inf, 0} */
        }
        if (x > o_threshold) return huge * huge;
        if (x < u_threshold) return twom1000 * twom1000;
    }
    if (hx > 0x3fd62e42u) {  /* |x| > 0.5 ln2 */
        if (hx < 0x3FF0A2B2u) {  /* and |x| < 1.5 ln2 */
            hi = xsb ? x + ln2hi : x - ln2hi;
            lo = xsb ? -ln2lo : ln2lo;
            k = 1 - xsb - xsb;
        } else {
            k = (int32_t)(invln2 * x + (xsb ? -0.5 : 0.5));
            t = (double)k;
            hi = x - t * ln2hi;
            lo = t * ln2lo;
        }
        x = hi - lo;
    } else if (hx < 0x3e300000u) {  /* |x| < 2**-28 */
        if (huge + x > one) return one + x;
    } else {
        k = 0;
    }
    t = x * x;
    c = x - t * (P1 + t * (P2 + t * (P3 + t * (P4 + t * P5))));
    if (k == 0) return one - (GBM_DIV(x * c, c - 2.0) - x);
    y = one - ((lo - GBM_DIV(x * c, 2.0 - c)) - hi);
    if (k >= -1021) return gbm_set_hi(y, gbm_hi(y) + (k << 20));
    return gbm_set_hi(y, gbm_hi(y) + ((k + 1000) << 20)) * twom1000;
}

/* ------------------------------------------------------------------ log */
GBM_HD double gbm_log(double x) {
    const double ln2_hi = 6.93147180369123816490e-01, ln2_lo = 1.90821492927058770002e-10;
    const double two54 = 1.80143985094819840000e+16;
    const double Lg1 = 6.666666666666735130e-01, Lg2 = 3.999999999940941908e-01, Lg3 = 2.857142874366239149e-01,
                 Lg4 = 2.222219843214978396e-01, Lg5 = 1.818357216161805012e-01, Lg6 = 1.531383769920937332e-01,
                 Lg7 = 1.479819860511658591e-01;
    double hfsq, f, s, z, R, w, t1, t2, dk;
    int32_t k = 0, hx = gbm_hi(x), i, j;
    const uint32_t lx = gbm_lo(x);
    if (hx < 0x00100000) {  /* x < 2**-1022 */
        if (((hx & 0x7fffffff) | (int32_t)lx) == 0) return -two54 / 0.0;  /* log(+-0) = -inf */
        if (hx < 0) return (x - x) / 0.0;                                  /* log(-#) = NaN */
        k -= 54;
        x *= two54;  /* subnormal: scale up */
        hx = gbm_hi(x);
    }
    if (hx >= 0x7ff00000) return x + x;
    k += (hx >> 20) - 1023;
    hx &= 0x000fffff;
    i = (hx + 0x95f64) & 0x100000;
    x = gbm_set_hi(x, hx | (i ^ 0x3ff00000));  /* x or x / 2 in [sqrt(2)/2, sqrt(2)) */
    k += (i >> 20);
    f = x - 1.0;
    if ((0x000fffff & (2 + hx)) < 3) {  /* |f| < 2**-20 */
        if (f == 0.0) {
            if (k == 0) return 0.0;
            dk = (double)k;
            return dk * ln2_hi + dk * ln2_lo;
        }
        R = f * f * (0.5 - 0.33333333333333333 * f);
        if (k == 0) return f - R;
        dk = (double)k;
        return dk * ln2_hi - ((R - dk * ln2_lo) - f);
    }
    s = GBM_DIV(f, 2.0 + f);
    dk = (double)k;
    z = s * s;
    i = hx - 0x6147a;
    w = z * z;
    j = 0x6b851 - hx;
    t1 = w * (Lg2 + w * (Lg4 + w * Lg6));
    t2 = z * (Lg1 + w * (Lg3 + w * (Lg5 + w * Lg7)));
    i |= j;
    R = t2 + t1;
    /* dk ln2_hi and dk ln2_lo, the two tails' common products, made once before the tails split
       (a warp whose lanes take both tails then issues them once) */
    const double dhi = dk * ln2_hi, dlo = dk * ln2_lo;
    if (i > 0) {
        hfsq = 0.5 * f * f;
        if (k == 0) return f - (hfsq - s * (hfsq + R));
        return dhi - ((hfsq - (s * (hfsq + R) + dlo)) - f);
    }
    if (k == 0) return f - s * (f - R);
    return dhi - ((s * (f - R) - dlo) - f);
}

/* ------------------------------------------------------------------ pow */
GBM_HD double gbm_pow(double x, double y) {
    /* bp, dp_h, dp_l of fdlibm's two-entry tables (k = 0, 1), picked by selects rather than an
       index (an indexed table lives in local memory on the device) */
    const double dp_h1 = 5.84962487220764160156e-01, dp_l1 = 1.35003920212974897128e-08;
    const double zero = 0.0, one = 1.0, two = 2.0, two53 = 9007199254740992.0, huge = 1.0e300, tiny = 1.0e-300;
    const double L1 = 5.99999999999994648725e-01, L2 = 4.28571428578550184252e-01, L3 = 3.33333329818377432918e-01,
                 L4 = 2.72728123808534006489e-01, L5 = 2.30660745775561754067e-01, L6 = 2.06975017800338417784e-01;
    const double P1 = 1.66666666666666019037e-01, P2 = -2.77777777770155933842e-03,
                 P3 = 6.61375632143793436117e-05, P4 = -1.65339022054652515390e-06,
                 P5 = 4.13813679705723846039e-08;
    const double lg2 = 6.93147180559945286227e-01, lg2_h = 6.93147182464599609375e-01,
                 lg2_l = -1.90465429995776804525e-09, ovt = 8.0085662595372944372e-17;
    const double cp = 9.61796693925975554329e-01, cp_h = 9.61796700954437255859e-01,
                 cp_l = -7.02846165095275826516e-09;
    const double ivln2 = 1.44269504088896338700e+00, ivln2_h = 1.44269502162933349609e+00,
                 ivln2_l = 1.92596299112661746887e-08;
    double z, ax, z_h, z_l, p_h, p_l, y1, t1, t2, r, s, t, u, v, w;
    int32_t i, j, k, yisint, n;
    int32_t hx = gbm_hi(x), hy = gbm_hi(y);
    const uint32_t lx = gbm_lo(x), ly = gbm_lo(y);
    int32_t ix = hx & 0x7fffffff;
    const int32_t iy = hy & 0x7fffffff;

    if ((iy | (int32_t)ly) == 0) return one;                 /* x**0 = 1 */
    if (hx == 0x3ff00000 && lx == 0) return one;            /* 1**y = 1 (C99) */
    if (ix > 0x7ff00000 || (ix == 0x7ff00000 && lx != 0) || iy > 0x7ff00000 || (iy == 0x7ff00000 && ly != 0))
        return x + y;                                        /* NaN */
    /* yisint: 0 not an integer, 1 odd, 2 even (only needed for x < 0) */
    yisint = 0;
    if (hx < 0) {
        if (iy >= 0x43400000) {
            yisint = 2;
        } else if (iy >= 0x3ff00000) {
            k = (iy >> 20) - 0x3ff;
            if (k > 20) {
                j = (int32_t)(ly >> (52 - k));
                if (((uint32_t)j << (52 - k)) == ly) yisint = 2 - (j & 1);
            } else if (ly == 0) {
                j = iy >> (20 - k);
                if ((j << (20 - k)) == iy) yisint = 2 - (j & 1);
            }
        }
    }
    if (ly == 0) {
        if (iy == 0x7ff00000) {  /* y = +-inf */
            if (((ix - 0x3ff00000) | (int32_t)lx) == 0) return one;  /* (-1)**+-inf = 1 (C99) */
            if (ix >= 0x3ff00000) return (hy >= 0) ? y : zero;
            return (hy < 0) ? -y : zero;
        }
        if (iy == 0x3ff00000) return (hy < 0) ? one / x : x;  /* y = +-1 */
        if (hy == 0x40000000) return x * x;                  /* y = 2 */
    }
    ax = gbm_fabs(x);
    if (lx == 0) {  /* x = +-0, +-inf, +-1 */
        if (ix == 0x7ff00000 || ix == 0 || ix == 0x3ff00000) {
            z = ax;
            if (hy < 0) z = one / z;
            if (hx < 0) {
                if (((ix - 0x3ff00000) | yisint) == 0)
                    z = (z - z) / (z - z);  /* (-1)**non-int */
                else if (yisint == 1)
                    z = -z;
            }
            return z;
        }
    }
    n = (int32_t)(((uint32_t)hx >> 31) - 1u);
    if ((n | yisint) == 0) return (x - x) / (x - x);  /* (x < 0)**non-int */
    s = one;
    if ((n | (yisint - 1)) == 0) s = -one;  /* (-ve)**odd */

    if (iy > 0x41e00000) {  /* |y| > 2**31 */
        if (iy > 0x43f00000) {
            if (ix <= 0x3fefffff) return (hy < 0) ? huge * huge : tiny * tiny;
            if (ix >= 0x3ff00000) return (hy > 0) ? huge * huge : tiny * tiny;
        }
        if (ix < 0x3fefffff) return (hy < 0) ? s * huge * huge : s * tiny * tiny;
        if (ix > 0x3ff00000) return (hy > 0) ? s * huge * huge : s * tiny * tiny;
        t = ax - one;
        w = (t * t) * (0.5 - t * (0.3333333333333333333333 - t * 0.25));
        u = ivln2_h * t;
        v = t * ivln2_l - w * ivln2;
        t1 = gbm_set_lo(u + v, 0);
        t2 = v - (t1 - u);
    } else {
        double ss, s2, s_h, s_l, t_h, t_l;
        n = 0;
        if (ix < 0x00100000) {  /* subnormal x */
            ax *= two53;
            n -= 53;
            ix = gbm_hi(ax);
        }
        n += ((ix) >> 20) - 0x3ff;
        j = ix & 0x000fffff;
        ix = j | 0x3ff00000;
        if (j <= 0x3988E)
            k = 0;  /* |x| < sqrt(3/2) */
        else if (j < 0xBB67A)
            k = 1;  /* |x| < sqrt(3) */
        else {
            k = 0;
            n += 1;
            ix -= 0x00100000;
        }
        ax = gbm_set_hi(ax, ix);
        const double bpk = k ? 1.5 : 1.0, dphk = k ? dp_h1 : 0.0, dplk = k ? dp_l1 : 0.0;
        u = ax - bpk;
        v = GBM_DIV(one, ax + bpk);
        ss = u * v;
        s_h = gbm_set_lo(ss, 0);
        t_h = gbm_make(((ix >> 1) | 0x20000000) + 0x00080000 + (k << 18), 0);
        t_l = ax - (t_h - bpk);
        s_l = v * ((u - s_h * t_h) - s_h * t_l);
        s2 = ss * ss;
        r = s2 * s2 * (L1 + s2 * (L2 + s2 * (L3 + s2 * (L4 + s2 * (L5 + s2 * L6)))));
        r += s_l * (s_h + ss);
        s2 = s_h * s_h;
        t_h = gbm_set_lo(3.0 + s2 + r, 0);
        t_l = r - ((t_h - 3.0) - s2);
        u = s_h * t_h;
        v = s_l * t_h + t_l * ss;
        p_h = gbm_set_lo(u + v, 0);
        p_l = v - (p_h - u);
        z_h = cp_h * p_h;
        z_l = cp_l * p_h + p_l * cp + dplk;
        t = (double)n;
        t1 = gbm_set_lo(((z_h + z_l) + dphk) + t, 0);
        t2 = z_l - (((t1 - t) - dphk) - z_h);
    }
    /* (y1 + y2) * (t1 + t2) */
    y1 = gbm_set_lo(y, 0);
    p_l = (y - y1) * t1 + y * t2;
    p_h = y1 * t1;
    z = p_l + p_h;
    j = gbm_hi(z);
    i = (int32_t)gbm_lo(z);
    if (j >= 0x40900000) {  /* z >= 1024 */
        if (((j - 0x40900000) | i) != 0) return s * huge * huge;
        if (p_l + ovt > z - p_h) return s * huge * huge;
    } else if ((j & 0x7fffffff) >= 0x4090cc00) {  /* z <= -1075 */
        if (((j - (int32_t)0xc090cc00) | i) != 0) return s * tiny * tiny;
        if (p_l <= z - p_h) return s * tiny * tiny;
    }
    /* 2**(p_h + p_l) */
    i = j & 0x7fffffff;
    k = (i >> 20) - 0x3ff;
    n = 0;
    if (i > 0x3fe00000) {  /* |z| > 0.5: n = [z + 0.5] */
        n = j + (0x00100000 >> (k + 1));
        k = ((n & 0x7fffffff) >> 20) - 0x3ff;
        t = gbm_make(n & ~(0x000fffff >> k), 0);
        n = ((n & 0x000fffff) | 0x00100000) >> (20 - k);
        if (j < 0) n = -n;
        p_h -= t;
    }
    t = gbm_set_lo(p_l + p_h, 0);
    u = t * lg2_h;
    v = (p_l - (t - p_h)) * lg2 + t * lg2_l;
    z = u + v;
    w = v - (z - u);
    t = z * z;
    t1 = z - t * (P1 + t * (P2 + t * (P3 + t * (P4 + t * P5))));
    r = GBM_DIV(z * t1, t1 - two) - (w + z * w);
    z = one - (r - z);
    j = gbm_hi(z);
    j += (n << 20);
    if ((j >> 20) <= 0)
        z = gbm_scale2(z, n);  /* subnormal result */
    else
        z = gbm_set_hi(z, j);
    return s * z;
}

/* ------------------------------------------------------------------ sin, cos */
GBM_HD double gbm_ksin(double x, double y, int iy) {
    const double S1 = -1.66666666666666324348e-01, S2 = 8.33333333332248946124e-03, S3 = -1.98412698298579493134e-04,
                 S4 = 2.75573137070700676789e-06, S5 = -2.50507602534068634195e-08, S6 = 1.58969099521155010221e-10;
    if ((gbm_hi(x) & 0x7fffffff) < 0x3e400000 && (int)x == 0) return x;  /* |x| < 2**-27, the sign of zero kept */
    const double z = x * x, v = z * x;
    const double r = S2 + z * (S3 + z * (S4 + z * (S5 + z * S6)));
    if (iy == 0) return x + v * (S1 + z * r);
    return x - ((z * (0.5 * y - v * r) - y) - v * S1);
}

GBM_HD double gbm_kcos(double x, double y) {
    const double C1 = 4.16666666666666019037e-02, C2 = -1.38888888888741095749e-03, C3 = 2.48015872894767294178e-05,
                 C4 = -2.75573143513906633035e-07, C5 = 2.08757232129817482790e-09, C6 = -1.13596475577881948265e-11;
    const int32_t ix = gbm_hi(x) & 0x7fffffff;
    if (ix < 0x3e400000 && (int)x == 0) return 1.0;
    const double z = x * x;
    const double r = z * (C1 + z * (C2 + z * (C3 + z * (C4 + z * (C5 + z * C6)))));
    if (ix < 0x3FD33333) return 1.0 - (0.5 * z - (z * r - x * y));
    const double qx = (ix > 0x3fe90000) ? 0.28125 : gbm_make(ix - 0x00200000, 0);
    const double hz = 0.5 * z - qx, a = 1.0 - qx;
    return a - (hz - (z * r - x * y));
}

/* x = n pi/2 + (y0 + y1), |x| < 2**19 pi/2: Cody-Waite with a 33 + 33 + 33 bit split of pi/2 */
GBM_HD int gbm_rem_pio2(double x, double *y0, double *y1) {
    const double invpio2 = 6.36619772367581382433e-01;
    const double pio2_1 = 1.57079632673412561417e+00, pio2_1t = 6.07710050650619224932e-11;
    const double pio2_2 = 6.07710050630396597660e-11, pio2_2t = 2.02226624879595063154e-21;
    const double pio2_3 = 2.02226624871116645580e-21, pio2_3t = 8.47842766036889956997e-32;
    const int32_t hx = gbm_hi(x), ix = hx & 0x7fffffff;
    if (ix <= 0x3fe921fb) {  /* |x| <= pi/4 */
        *y0 = x;
        *y1 = 0.0;
        return 0;
    }
    const double t = gbm_fabs(x);
    const int32_t n = (int32_t)(t * invpio2 + 0.5);
    const double fn = (double)n;
    double r = t - fn * pio2_1, w = fn * pio2_1t;
    double y = r - w;
    const int32_t j = ix >> 20;
    int32_t i = j - ((gbm_hi(y) >> 20) & 0x7ff);
    if (i > 16) {  /* a second iteration: 118 bits */
        double tt = r;
        w = fn * pio2_2;
        r = tt - w;
        w = fn * pio2_2t - ((tt - r) - w);
        y = r - w;
        i = j - ((gbm_hi(y) >> 20) & 0x7ff);
        if (i > 49) {  /* a third: 151 bits */
            tt = r;
            w = fn * pio2_3;
            r = tt - w;
            w = fn * pio2_3t - ((tt - r) - w);
            y = r - w;
        }
    }
    double y1v = (r - y) - w;
    if (hx < 0) {
        *y0 = -y;
        *y1 = -y1v;
        return -n;
    }
    *y0 = y;
    *y1 = y1v;
    return n;
}

GBM_HD double gbm_sin(double x) {
    const int32_t ix = gbm_hi(x) & 0x7fffffff;
    if (ix >= 0x7ff00000) return x - x;
    double y0, y1;
    const int n = gbm_rem_pio2(x, &y0, &y1);
    if (n == 0 && ix <= 0x3fe921fb) return gbm_ksin(x, 0.0, 0);
    switch (n & 3) {
        case 0: return gbm_ksin(y0, y1, 1);
        case 1: return gbm_kcos(y0, y1);
        case 2: return -gbm_ksin(y0, y1, 1);
        default: return -gbm_kcos(y0, y1);
    }
}

GBM_HD double gbm_cos(double x) {
    const int32_t ix = gbm_hi(x) & 0x7fffffff;
    if (ix >= 0x7ff00000) return x - x;
    double y0, y1;
    const int n = gbm_rem_pio2(x, &y0, &y1);
    if (n == 0 && ix <= 0x3fe921fb) return gbm_kcos(x, 0.0);
    switch (n & 3) {
        case 0: return gbm_kcos(y0, y1);
        case 1: return -gbm_ksin(y0, y1, 1);
        case 2: return -gbm_kcos(y0, y1);
        default: return gbm_ksin(y0, y1, 1);
    }
}

#endif /* GBMATH_H */
