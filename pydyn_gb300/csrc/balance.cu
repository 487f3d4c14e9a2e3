// Meteo_Setup_Mass on the device: the mass change the surface-pressure tendency asks of every
// cell, the check of the column-integrated convergence against it, and the balancing of the
// horizontal fluxes -- region 1 by the doubly periodic Poisson correction of each level's
// residual divergence, a child by its parent cells' direct Poisson matrices after its fluxes
// have been matched to its parent's.
//
// The Poisson solve is a separable discrete Fourier transform in float64: along i, then along
// j, division by the periodic 5-point Laplacian's eigenvalues, and back.  The reference calls
// FFTW (or NumPy's FFT); neither's operation order is reproduced, so the balanced fluxes agree
// with the reference's to rounding (a few ulp of the corrections), not bitwise.  Everything
// around the transform is the reference's element statement in its order.
//
// Reference: pydyn balance.py:76-94 (fill_mass_change, check_mass_balance), :97-104
// (poisson_factor), :107-124 (NumpyPoisson), :183-199 (poisson_correction,
// balance_mass_fluxes), :202-219 (setup_mass); zoom_meteo.py:87-133 (match_cell_sum,
// match_u_sum, match_v_sum), :135-181 (PoissonDirect, balance_mass_fluxes_child).
#include "gb_common.cuh"

namespace {

constexpr double GRAV = 9.80665;

__device__ __forceinline__ double &E3(const DV &v, int64_t i, int64_t j, int64_t l) {
    return v.p[i * v.s0 + j * v.s1 + l * v.s2];
}
__device__ __forceinline__ double E2(const DV &v, int64_t i, int64_t j) { return v.p[i * v.s0 + j * v.s1]; }

unsigned grid_for(int64_t n, int threads) { return (unsigned)((n + threads - 1) / threads); }

// ------------------------------------------------------------------ mass change, residual
// dm_dt(i, j, l) = ((|db(l)| (sp2 - sp1) / g) area(j)) / dt
__global__ void k_fill_mass_change(DV dm, DV sp1, DV sp2, const double *db, const double *area, double dt,
                                   int im, int jm, int lm) {
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (int64_t)im * jm * lm) return;
    const int l = (int)(t % lm), j = (int)((t / lm) % jm), i = (int)(t / ((int64_t)lm * jm));
    const double d = fabs(db[l]) * (E2(sp2, i, j) - E2(sp1, i, j)) / GRAV;
    E3(dm, i, j, l) = (d * area[j]) / dt;
}

// the residual divergence of each cell and level: convergence(pu, pv) + pw(l) - pw(l+1) - dm_dt
__global__ void k_residual(DV pu, DV pv, DV pw, DV dm, double *res, int im, int jm, int lm) {
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (int64_t)im * jm * lm) return;
    const int l = (int)(t % lm), j = (int)((t / lm) % jm), i = (int)(t / ((int64_t)lm * jm));
    const double c = E3(pu, i, j, l) - E3(pu, i + 1, j, l) + E3(pv, i, j, l) - E3(pv, i, j + 1, l);
    res[t] = c + E3(pw, i, j, l) - E3(pw, i, j, l + 1) - E3(dm, i, j, l);  // (i, j, l), l fastest
}

// ------------------------------------------------------------------ CheckMassBalance
// diff(i, j) = (conv(seqsum pu, seqsum pv) g / area(j) - (sp2 - sp1) / dt) / ((sp1 + sp2) / 2)
__global__ void k_balance_diff(DV pu, DV pv, DV sp1, DV sp2, const double *area, double dt, double *diff, int im,
                               int jm, int lm) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= im * jm) return;
    const int i = t / jm, j = t % jm;
    double u0 = E3(pu, i, j, 0), u1 = E3(pu, i + 1, j, 0), v0 = E3(pv, i, j, 0), v1 = E3(pv, i, j + 1, 0);
    for (int l = 1; l < lm; ++l) {  // seqsum: the levels in order
        u0 = u0 + E3(pu, i, j, l);
        u1 = u1 + E3(pu, i + 1, j, l);
        v0 = v0 + E3(pv, i, j, l);
        v1 = v1 + E3(pv, i, j + 1, l);
    }
    const double d = (u0 - u1 + v0 - v1) * GRAV / area[j];
    const double a = E2(sp1, i, j), b = E2(sp2, i, j);
    diff[t] = (d - (b - a) / dt) / ((a + b) / 2.0);
}

// one block: out = (rms, max |diff|) of n values, summed in a fixed tree order
__global__ void k_balance_stats(const double *diff, int n, double *out) {
    __shared__ double ssum[1024], smax[1024];
    double s = 0.0, mx = 0.0;
    for (int k = threadIdx.x; k < n; k += blockDim.x) {
        const double d = diff[k];
        s = s + d * d;
        mx = fmax(mx, fabs(d));
    }
    ssum[threadIdx.x] = s;
    smax[threadIdx.x] = mx;
    __syncthreads();
    for (int w = blockDim.x / 2; w > 0; w >>= 1) {
        if (threadIdx.x < w) {
            ssum[threadIdx.x] = ssum[threadIdx.x] + ssum[threadIdx.x + w];
            smax[threadIdx.x] = fmax(smax[threadIdx.x], smax[threadIdx.x + w]);
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        out[0] = sqrt(ssum[0] / (double)n);
        out[1] = smax[0];
    }
}

// ------------------------------------------------------------------ the periodic Poisson solve
// tw: cos, sin of 2 pi t / N for t = 0..N-1 (2N doubles); complex arrays interleaved (re, im)
// forward along i: A(k, j, l) = sum_i r(i, j, l) exp(-2 pi i k i / im)
__global__ void k_dft_i(const double *r, const double *tw, double *A, int im, int jm, int lm) {
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (int64_t)im * jm * lm) return;
    const int l = (int)(t % lm), j = (int)((t / lm) % jm), k = (int)(t / ((int64_t)lm * jm));
    double re = 0.0, ig = 0.0;
    int p = 0;  // (k i) mod im
    for (int i = 0; i < im; ++i) {
        const double x = r[((int64_t)i * jm + j) * lm + l];
        re = re + x * tw[p];
        ig = ig - x * tw[im + p];
        p += k;
        if (p >= im) p -= im;
    }
    A[2 * t] = re;
    A[2 * t + 1] = ig;
}

// forward along j, then X / fac (the real and imaginary parts divided apart, X(0, 0) = 0)
__global__ void k_dft_j_divide(const double *A, const double *tw, const double *fac, double *X, int im, int jm,
                               int lm) {
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (int64_t)im * jm * lm) return;
    const int l = (int)(t % lm), k2 = (int)((t / lm) % jm), k1 = (int)(t / ((int64_t)lm * jm));
    double re = 0.0, ig = 0.0;
    int p = 0;
    for (int j = 0; j < jm; ++j) {
        const int64_t s = ((int64_t)k1 * jm + j) * lm + l;
        const double ar = A[2 * s], ai = A[2 * s + 1], c = tw[p], sn = tw[jm + p];
        re = re + (ar * c + ai * sn);  // (ar + i ai)(c - i sn)
        ig = ig + (ai * c - ar * sn);
        p += k2;
        if (p >= jm) p -= jm;
    }
    const double f = fac[(int64_t)k1 * jm + k2];
    X[2 * t] = (k1 == 0 && k2 == 0) ? 0.0 : re / f;
    X[2 * t + 1] = (k1 == 0 && k2 == 0) ? 0.0 : ig / f;
}

// backward along j: B(k1, j, l) = sum_k2 X(k1, k2, l) exp(+2 pi i k2 j / jm)
__global__ void k_idft_j(const double *X, const double *tw, double *B, int im, int jm, int lm) {
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (int64_t)im * jm * lm) return;
    const int l = (int)(t % lm), j = (int)((t / lm) % jm), k1 = (int)(t / ((int64_t)lm * jm));
    double re = 0.0, ig = 0.0;
    int p = 0;
    for (int k2 = 0; k2 < jm; ++k2) {
        const int64_t s = ((int64_t)k1 * jm + k2) * lm + l;
        const double xr = X[2 * s], xi = X[2 * s + 1], c = tw[p], sn = tw[jm + p];
        re = re + (xr * c - xi * sn);  // (xr + i xi)(c + i sn)
        ig = ig + (xi * c + xr * sn);
        p += j;
        if (p >= jm) p -= jm;
    }
    B[2 * t] = re;
    B[2 * t + 1] = ig;
}

// backward along i, the real part: psi(i, j, l) = Re sum_k1 B(k1, j, l) exp(+2 pi i k1 i / im) / (im jm)
__global__ void k_idft_i_real(const double *B, const double *tw, double *psi, int im, int jm, int lm) {
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (int64_t)im * jm * lm) return;
    const int l = (int)(t % lm), j = (int)((t / lm) % jm), i = (int)(t / ((int64_t)lm * jm));
    double re = 0.0;
    int p = 0;
    for (int k1 = 0; k1 < im; ++k1) {
        const int64_t s = ((int64_t)k1 * jm + j) * lm + l;
        re = re + (B[2 * s] * tw[p] - B[2 * s + 1] * tw[im + p]);
        p += i;
        if (p >= im) p -= im;
    }
    psi[t] = re / (double)((int64_t)im * jm);
}

// the corrections: u = psi(i) - psi(i-1) across every x face (periodic), gauged by face 0; v the
// same across y faces; added to pu, pv
__global__ void k_correct(const double *psi, DV pu, DV pv, int im, int jm, int lm) {
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const int64_t nu = (int64_t)(im + 1) * jm * lm, nv = (int64_t)im * (jm + 1) * lm;
    auto P = [&](int i, int j, int l) { return psi[((int64_t)i * jm + j) * lm + l]; };
    if (t < nu) {
        const int l = (int)(t % lm), j = (int)((t / lm) % jm), i = (int)(t / ((int64_t)lm * jm));
        const double u = (i < im ? P(i, j, l) : P(0, j, l)) - P(i > 0 ? i - 1 : im - 1, j, l);
        const double u0 = P(0, j, l) - P(im - 1, j, l);
        E3(pu, i, j, l) = E3(pu, i, j, l) + (u - u0);
    } else if (t < nu + nv) {
        const int64_t s = t - nu;
        const int l = (int)(s % lm), j = (int)((s / lm) % (jm + 1)), i = (int)(s / ((int64_t)lm * (jm + 1)));
        const double v = (j < jm ? P(i, j, l) : P(i, 0, l)) - P(i, j > 0 ? j - 1 : jm - 1, l);
        const double v0 = P(i, 0, l) - P(i, jm - 1, l);
        E3(pv, i, j, l) = E3(pv, i, j, l) + (v - v0);
    }
}

// ------------------------------------------------------------------ a child: Match 'sum'
// kind 0: x faces (Match_u), 1: y faces (Match_v), 2: cells (Match_cell), every level; a thread
// per (parent face or cell, level)
struct MatchArgs {
    DV pg, tg;
    int kind, ri, rj, ci1, ci2, cj1, cj2, lm;
};

__global__ void k_match_sum(MatchArgs M) {
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const int ni = M.kind == 0 ? M.ci2 - M.ci1 + 2 : M.ci2 - M.ci1 + 1;
    const int nj = M.kind == 1 ? M.cj2 - M.cj1 + 2 : M.cj2 - M.cj1 + 1;
    if (t >= (int64_t)ni * nj * M.lm) return;
    const int l = (int)(t % M.lm), a = (int)((t / M.lm) % ni), b = (int)(t / ((int64_t)M.lm * ni));
    if (M.kind == 0) {  // parent x face ci = ci1 - 1 + a at row cj = cj1 + b: the rj child faces along j
        const int ci = M.ci1 - 1 + a, cj = M.cj1 + b, fi = a * M.ri, fj = b * M.rj;
        double s = E3(M.tg, fi, fj, l);
        for (int q = 1; q < M.rj; ++q) s = s + E3(M.tg, fi, fj + q, l);
        const double add = (E3(M.pg, ci, cj - 1, l) - s) / M.rj;
        for (int q = 0; q < M.rj; ++q) E3(M.tg, fi, fj + q, l) = E3(M.tg, fi, fj + q, l) + add;
    } else if (M.kind == 1) {  // parent y face cj = cj1 - 1 + b at column ci = ci1 + a
        const int ci = M.ci1 + a, cj = M.cj1 - 1 + b, fi = a * M.ri, fj = b * M.rj;
        double s = E3(M.tg, fi, fj, l);
        for (int q = 1; q < M.ri; ++q) s = s + E3(M.tg, fi + q, fj, l);
        const double add = (E3(M.pg, ci - 1, cj, l) - s) / M.ri;
        for (int q = 0; q < M.ri; ++q) E3(M.tg, fi + q, fj, l) = E3(M.tg, fi + q, fj, l) + add;
    } else {  // parent cell: the block's sum in column-major order (i fastest)
        const int ci = M.ci1 + a, cj = M.cj1 + b, fi = a * M.ri, fj = b * M.rj;
        double s = E3(M.tg, fi, fj, l);
        for (int q = 1; q < M.ri * M.rj; ++q) s = s + E3(M.tg, fi + q % M.ri, fj + q / M.ri, l);
        const double add = (E3(M.pg, ci - 1, cj - 1, l) - s) / (M.rj * M.ri);
        for (int q = 0; q < M.ri * M.rj; ++q)
            E3(M.tg, fi + q % M.ri, fj + q / M.ri, l) = E3(M.tg, fi + q % M.ri, fj + q / M.ri, l) + add;
    }
}

// ------------------------------------------------------------------ a child: the direct solve
// thread per level: every parent cell in the Fortran order (cj outer, ci inner), its block's
// residual vector (column-major) through the direct matrices, the corrections added to the
// block's faces (a face between two blocks takes both, in that order)
struct DirectArgs {
    DV pu, pv;
    const double *res;  // (im, jm, lm), l fastest
    const double *mu, *mv;  // m_to_u ((ri+1) rj x n), m_to_v (ri (rj+1) x n), column-major
    int im, jm, lm, ri, rj, ci1, ci2, cj1, cj2;
};

__global__ void k_balance_direct(DirectArgs D) {
    const int l = blockIdx.x * blockDim.x + threadIdx.x;
    if (l >= D.lm) return;
    const int n = D.ri * D.rj, nu = (D.ri + 1) * D.rj, nv = D.ri * (D.rj + 1);
    double vec[64];
    for (int cj = D.cj1; cj <= D.cj2; ++cj)
        for (int ci = D.ci1; ci <= D.ci2; ++ci) {
            const int fi = (ci - D.ci1) * D.ri, fj = (cj - D.cj1) * D.rj;
            for (int k = 0; k < n; ++k)
                vec[k] = D.res[((int64_t)(fi + k % D.ri) * D.jm + fj + k / D.ri) * D.lm + l];
            for (int r = 0; r < nu; ++r) {  // u face r: (r % (ri+1), r / (ri+1)) of the block
                double u = 0.0;
                for (int k = 0; k < n; ++k) u = u + D.mu[(int64_t)k * nu + r] * vec[k];
                const int a = r % (D.ri + 1), b = r / (D.ri + 1);
                E3(D.pu, fi + a, fj + b, l) = E3(D.pu, fi + a, fj + b, l) + u;
            }
            for (int r = 0; r < nv; ++r) {  // v face r: (r % ri, r / ri)
                double v = 0.0;
                for (int k = 0; k < n; ++k) v = v + D.mv[(int64_t)k * nv + r] * vec[k];
                const int a = r % D.ri, b = r / D.ri;
                E3(D.pv, fi + a, fj + b, l) = E3(D.pv, fi + a, fj + b, l) + v;
            }
        }
}

int dims_of(const gb_view *pu, const gb_view *pv, const gb_view *pw, int *im, int *jm, int *lm,
            const gb_view *dm = nullptr) {
    *im = (int)pv->n[0];
    *jm = (int)pu->n[1];
    *lm = (int)pu->n[2];
    if (pu->n[0] != *im + 1 || pv->n[1] != *jm + 1 || pv->n[2] != *lm || (pw && (pw->n[0] != *im ||
                                                                             pw->n[1] != *jm || pw->n[2] != *lm + 1))) {
        gb_set_error("balance: pu (im+1, jm, lm), pv (im, jm+1, lm), pw (im, jm, lm+1) disagree");
        return GB_EARG;
    }
    if (dm && (dm->n[0] != *im || dm->n[1] != *jm || dm->n[2] != *lm)) {
        gb_set_error("balance: dm_dt is not (im, jm, lm)");
        return GB_EARG;
    }
    return GB_OK;
}

}  // namespace

extern "C" int gb_fill_mass_change(gb_ctx *ctx, const gb_view *dm_dt, const gb_view *sp1, const gb_view *sp2,
                                   const double *levi_db, const double *area, double dt_sec) {
    if (!ctx || !dm_dt || !sp1 || !sp2 || !levi_db || !area) return GB_EARG;
    const int im = (int)dm_dt->n[0], jm = (int)dm_dt->n[1], lm = (int)dm_dt->n[2];
    if (sp1->n[0] != im || sp1->n[1] != jm || sp2->n[0] != im || sp2->n[1] != jm) {
        gb_set_error("gb_fill_mass_change: sp1, sp2 are not (im, jm) of dm_dt");
        return GB_EARG;
    }
    const int64_t n = (int64_t)im * jm * lm;
    if (n <= 0) return GB_OK;
    k_fill_mass_change<<<grid_for(n, 256), 256, 0, ctx->stream>>>(dv(dm_dt), dv(sp1), dv(sp2), levi_db, area, dt_sec,
                                                                  im, jm, lm);
    return gb_after_launch(ctx, "fill_mass_change");
}

extern "C" int gb_mass_check(gb_ctx *ctx, const gb_view *pu, const gb_view *pv, const gb_view *sp1,
                             const gb_view *sp2, const double *area, double dt_sec, double *out) {
    if (!ctx || !pu || !pv || !sp1 || !sp2 || !area || !out) return GB_EARG;
    int im, jm, lm;
    if (int rc = dims_of(pu, pv, nullptr, &im, &jm, &lm)) return rc;
    if (im <= 0 || jm <= 0 || lm <= 0) return GB_EARG;
    if (sp1->n[0] != im || sp1->n[1] != jm || sp2->n[0] != im || sp2->n[1] != jm) {
        gb_set_error("gb_mass_check: sp1, sp2 are not (im, jm)");
        return GB_EARG;
    }
    double *diff = gb_work(ctx, (size_t)im * jm * sizeof(double));
    if (!diff) return GB_ECUDA;
    k_balance_diff<<<grid_for((int64_t)im * jm, 128), 128, 0, ctx->stream>>>(dv(pu), dv(pv), dv(sp1), dv(sp2), area,
                                                                             dt_sec, diff, im, jm, lm);
    if (int rc = gb_after_launch(ctx, "mass_check")) return rc;
    k_balance_stats<<<1, 1024, 0, ctx->stream>>>(diff, im * jm, out);
    return gb_after_launch(ctx, "mass_check_stats");
}

extern "C" int gb_balance_fft(gb_ctx *ctx, const gb_view *pu, const gb_view *pv, const gb_view *pw,
                              const gb_view *dm_dt, const double *tw_i, const double *tw_j, const double *fac) {
    if (!ctx || !pu || !pv || !pw || !dm_dt || !tw_i || !tw_j || !fac) return GB_EARG;
    int im, jm, lm;
    if (int rc = dims_of(pu, pv, pw, &im, &jm, &lm, dm_dt)) return rc;
    const int64_t n = (int64_t)im * jm * lm;
    if (n <= 0) return GB_OK;
    // work: the residual (n), two complex arrays (2n each), psi in the residual's place
    double *w = gb_work(ctx, (size_t)5 * n * sizeof(double));
    if (!w) return GB_ECUDA;
    double *res = w, *A = w + n, *X = w + 3 * n;
    const unsigned g = grid_for(n, 256);
    k_residual<<<g, 256, 0, ctx->stream>>>(dv(pu), dv(pv), dv(pw), dv(dm_dt), res, im, jm, lm);
    if (int rc = gb_after_launch(ctx, "balance_residual")) return rc;
    k_dft_i<<<g, 256, 0, ctx->stream>>>(res, tw_i, A, im, jm, lm);
    if (int rc = gb_after_launch(ctx, "balance_dft_i")) return rc;
    k_dft_j_divide<<<g, 256, 0, ctx->stream>>>(A, tw_j, fac, X, im, jm, lm);
    if (int rc = gb_after_launch(ctx, "balance_dft_j")) return rc;
    k_idft_j<<<g, 256, 0, ctx->stream>>>(X, tw_j, A, im, jm, lm);
    if (int rc = gb_after_launch(ctx, "balance_idft_j")) return rc;
    k_idft_i_real<<<g, 256, 0, ctx->stream>>>(A, tw_i, res, im, jm, lm);
    if (int rc = gb_after_launch(ctx, "balance_idft_i")) return rc;
    const int64_t faces = (int64_t)(im + 1) * jm * lm + (int64_t)im * (jm + 1) * lm;
    k_correct<<<grid_for(faces, 256), 256, 0, ctx->stream>>>(res, dv(pu), dv(pv), im, jm, lm);
    return gb_after_launch(ctx, "balance_correct");
}

extern "C" int gb_match_sum(gb_ctx *ctx, int kind, const gb_view *parent, const gb_view *child, int ri, int rj,
                            int ci1, int ci2, int cj1, int cj2) {
    if (!ctx || !parent || !child || kind < 0 || kind > 2 || ri < 1 || rj < 1 || ci2 < ci1 || cj2 < cj1) return GB_EARG;
    const int ni = ci2 - ci1 + 1, nj = cj2 - cj1 + 1;
    const int64_t want0 = kind == 0 ? (int64_t)ni * ri + 1 : (int64_t)ni * ri;
    const int64_t want1 = kind == 1 ? (int64_t)nj * rj + 1 : (int64_t)nj * rj;
    if (child->n[0] != want0 || child->n[1] != want1 || parent->n[2] != child->n[2] || ci1 < 1 || cj1 < 1 ||
        parent->n[0] < (kind == 0 ? ci2 + 1 : ci2) || parent->n[1] < (kind == 1 ? cj2 + 1 : cj2)) {
        gb_set_error("gb_match_sum: the child's extents are not its footprint times its refinement");
        return GB_EARG;
    }
    MatchArgs M{dv(parent), dv(child), kind, ri, rj, ci1, ci2, cj1, cj2, (int)child->n[2]};
    const int64_t n = (int64_t)(kind == 0 ? ni + 1 : ni) * (kind == 1 ? nj + 1 : nj) * M.lm;
    if (n <= 0) return GB_OK;
    k_match_sum<<<grid_for(n, 128), 128, 0, ctx->stream>>>(M);
    return gb_after_launch(ctx, "match_sum");
}

extern "C" int gb_balance_direct(gb_ctx *ctx, const gb_view *pu, const gb_view *pv, const gb_view *pw,
                                 const gb_view *dm_dt, const double *m_to_u, const double *m_to_v, int ri, int rj,
                                 int ci1, int ci2, int cj1, int cj2) {
    if (!ctx || !pu || !pv || !pw || !dm_dt || !m_to_u || !m_to_v || ri < 1 || rj < 1) return GB_EARG;
    if (ri * rj > 64) {
        gb_set_error("gb_balance_direct: at most 64 child cells per parent cell");
        return GB_EARG;
    }
    int im, jm, lm;
    if (int rc = dims_of(pu, pv, pw, &im, &jm, &lm, dm_dt)) return rc;
    if ((ci2 - ci1 + 1) * ri != im || (cj2 - cj1 + 1) * rj != jm) {
        gb_set_error("gb_balance_direct: the region is not its footprint times its refinement");
        return GB_EARG;
    }
    const int64_t n = (int64_t)im * jm * lm;
    double *res = gb_work(ctx, (size_t)n * sizeof(double));
    if (!res) return GB_ECUDA;
    k_residual<<<grid_for(n, 256), 256, 0, ctx->stream>>>(dv(pu), dv(pv), dv(pw), dv(dm_dt), res, im, jm, lm);
    if (int rc = gb_after_launch(ctx, "balance_residual")) return rc;
    DirectArgs D{dv(pu), dv(pv), res, m_to_u, m_to_v, im, jm, lm, ri, rj, ci1, ci2, cj1, cj2};
    k_balance_direct<<<grid_for(lm, 32), 32, 0, ctx->stream>>>(D);
    return gb_after_launch(ctx, "balance_direct");
}
