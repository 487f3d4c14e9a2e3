// The parent <-> child exchange of the zoom tree, one fused kernel per body, indices in the
// Fortran bounds the state is declared with (m, tracers (-1:im+2, -1:jm+2, 1:lm[, 1:nt]);
// am, bm, cm (0:im+1, 0:jm+1, 0:lm+1)).
// Reference: pydyn zoom/exchange.py:17-258 (put_xedges, put_yedges, compress / uncompress,
// mix_edges, update_parent), zoom/massflow.py:334-428 (_coarsen_block, coarsen_ambm).
#include "gb_common.cuh"

namespace {

struct RA {            // one region's arrays, whole (halo'd)
    DV m, q[4];        // q: rm, rxm, rym, rzm
    DV am, bm, cm;
    int im, jm, lm, nt;
};

__device__ __forceinline__ double &Mc(const RA &r, int i, int j, int l) {  // m(i, j, l)
    return r.m.p[(int64_t)(i + 1) * r.m.s0 + (int64_t)(j + 1) * r.m.s1 + (int64_t)(l - 1) * r.m.s2];
}
__device__ __forceinline__ double &Qc(const RA &r, int w, int i, int j, int l, int t) {  // q(i, j, l, t+1)
    const DV &v = r.q[w];
    return v.p[(int64_t)(i + 1) * v.s0 + (int64_t)(j + 1) * v.s1 + (int64_t)(l - 1) * v.s2 + (int64_t)t * v.s3];
}
__device__ __forceinline__ double &Fc(const DV &v, int i, int j, int l) {  // am / bm / cm (i, j, l)
    return v.p[(int64_t)i * v.s0 + (int64_t)j * v.s1 + (int64_t)l * v.s2];
}
// field f of a region: 0 = m, 1..4 = rm, rxm, rym, rzm (tracer t)
__device__ __forceinline__ double &Xc(const RA &r, int f, int i, int j, int l, int t) {
    return f == 0 ? Mc(r, i, j, l) : Qc(r, f - 1, i, j, l, t);
}

static RA ra(const gb_view *v) {  // v[0..7]: m, rm, rxm, rym, rzm, am, bm, cm
    RA r;
    r.m = dv(&v[0]);
    for (int w = 0; w < 4; ++w) r.q[w] = dv(&v[1 + w]);
    r.am = dv(&v[5]); r.bm = dv(&v[6]); r.cm = dv(&v[7]);
    r.im = (int)v[0].n[0] - 4; r.jm = (int)v[0].n[1] - 4; r.lm = (int)v[0].n[2]; r.nt = (int)v[1].n[3];
    return r;
}

static int grid_for(int64_t total) {
    int64_t b = (total + 127) / 128;
    return (int)(b < 1 ? 1 : b);
}

// ------------------------------------------------------------------ put_xedges / put_yedges
// One thread per (child row jc, level lc, field f, tracer t): the parent's cells beside and on the
// child's x walls, scaled by 1/(yr zr) (outside) and 1/(xr yr zr) (inside; slopes: 1/(yr zr)),
// into the child's halo cell and its xr interface cells at each wall (exchange.py:17-60).
__global__ void k_put_xedges(RA P, RA C, int ib, int ie, int jbeg, int lbeg, int xr, int yr, int zr, double yzref,
                             double xyzref, int nfield) {
    int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    const int jmc = C.jm, lmc = C.lm;
    const int64_t per = (int64_t)jmc * lmc;
    if (k >= per * nfield) return;
    const int ft = (int)(k / per), rest = (int)(k % per);
    const int jc = rest / lmc + 1, lc = rest % lmc + 1;
    const int f = ft == 0 ? 0 : 1 + (ft - 1) / C.nt, t = ft == 0 ? 0 : (ft - 1) % C.nt;
    const int jp = jbeg + (jc - 1) / yr, lp = lbeg + (lc - 1) / zr;
    const double inner = (f == 0 || f == 1) ? xyzref : yzref;
    const double toc0 = Xc(P, f, ib - 1, jp, lp, t) * yzref;
    const double toc1 = Xc(P, f, ib, jp, lp, t) * inner;
    const double tocm = Xc(P, f, ie, jp, lp, t) * inner;
    const double tocm1 = Xc(P, f, ie + 1, jp, lp, t) * yzref;
    Xc(C, f, 0, jc, lc, t) = toc0;
    Xc(C, f, C.im + 1, jc, lc, t) = tocm1;
    for (int i = 1; i <= xr; ++i) {
        Xc(C, f, i, jc, lc, t) = toc1;
        Xc(C, f, C.im + 1 - i, jc, lc, t) = tocm;
    }
}

__global__ void k_put_yedges(RA P, RA C, int jb, int je, int ibeg, int lbeg, int xr, int yr, int zr, double xzref,
                             double xyzref, int nfield) {
    int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    const int imc = C.im, lmc = C.lm;
    const int64_t per = (int64_t)imc * lmc;
    if (k >= per * nfield) return;
    const int ft = (int)(k / per), rest = (int)(k % per);
    const int ic = rest / lmc + 1, lc = rest % lmc + 1;
    const int f = ft == 0 ? 0 : 1 + (ft - 1) / C.nt, t = ft == 0 ? 0 : (ft - 1) % C.nt;
    int ip = (ibeg - 1 + (ic - 1) / xr) % P.im;
    if (ip < 0) ip += P.im;
    ip += 1;
    const int lp = lbeg + (lc - 1) / zr;
    const double inner = (f == 0 || f == 1) ? xyzref : xzref;
    const double toc0 = Xc(P, f, ip, jb - 1, lp, t) * xzref;
    const double toc1 = Xc(P, f, ip, jb, lp, t) * inner;
    const double tocm = Xc(P, f, ip, je, lp, t) * inner;
    const double tocm1 = Xc(P, f, ip, je + 1, lp, t) * xzref;
    Xc(C, f, ic, 0, lc, t) = toc0;
    Xc(C, f, ic, C.jm + 1, lc, t) = tocm1;
    for (int j = 1; j <= yr; ++j) {
        Xc(C, f, ic, j, lc, t) = toc1;
        Xc(C, f, ic, C.jm + 1 - j, lc, t) = tocm;
    }
}

// ------------------------------------------------------------------ compress / uncompress
// x: one thread per (row j in js..je, level l in ls..le, field, tracer) (exchange.py:108-141).
__global__ void k_compress_x(RA R, int xr, int js, int je, int ls, int le, int nfield) {
    int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    const int nj = je - js + 1, nl = le - ls + 1;
    const int64_t per = (int64_t)nj * nl;
    if (nj <= 0 || nl <= 0 || k >= per * nfield) return;
    const int ft = (int)(k / per), rest = (int)(k % per);
    const int j = js + rest / nl, l = ls + rest % nl;
    const int f = ft == 0 ? 0 : 1 + (ft - 1) / R.nt, t = ft == 0 ? 0 : (ft - 1) % R.nt;
    const int imr = R.im;
    if (f <= 1) {  // m and rm: the interface cells' seqsum into the edge cell
        double s = Xc(R, f, 1, j, l, t);
        for (int i = 2; i <= xr; ++i) s = s + Xc(R, f, i, j, l, t);
        Xc(R, f, xr, j, l, t) = s;
        double e = Xc(R, f, imr - xr + 1, j, l, t);
        for (int i = imr - xr + 2; i <= imr; ++i) e = e + Xc(R, f, i, j, l, t);
        Xc(R, f, imr - xr + 1, j, l, t) = e;
    }
    Xc(R, f, xr - 1, j, l, t) = Xc(R, f, 0, j, l, t);
    Xc(R, f, imr - xr + 2, j, l, t) = Xc(R, f, imr + 1, j, l, t);
}

__global__ void k_uncompress_x(RA R, int xr, int js, int je, int ls, int le, int nfield) {
    int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    const int nj = je - js + 1, nl = le - ls + 1;
    const int64_t per = (int64_t)nj * nl;
    if (nj <= 0 || nl <= 0 || k >= per * nfield) return;
    const int ft = (int)(k / per), rest = (int)(k % per);
    const int j = js + rest / nl, l = ls + rest % nl;
    const int f = ft == 0 ? 0 : 1 + (ft - 1) / R.nt, t = ft == 0 ? 0 : (ft - 1) % R.nt;
    const int imr = R.im;
    const double w = div_ip(Xc(R, f, xr, j, l, t), (double)xr);
    for (int i = 1; i <= xr; ++i) Xc(R, f, i, j, l, t) = w;
    const double e = div_ip(Xc(R, f, imr - xr + 1, j, l, t), (double)xr);
    for (int i = imr - xr + 1; i <= imr; ++i) Xc(R, f, i, j, l, t) = e;
}

// y: one thread per (column i in is..ie, level l in ls..le, field, tracer) (exchange.py:144-175).
__global__ void k_compress_y(RA R, int yr, int is, int ie, int ls, int le, int nfield) {
    int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    const int ni = ie - is + 1, nl = le - ls + 1;
    const int64_t per = (int64_t)ni * nl;
    if (ni <= 0 || nl <= 0 || k >= per * nfield) return;
    const int ft = (int)(k / per), rest = (int)(k % per);
    const int i = is + rest / nl, l = ls + rest % nl;
    const int f = ft == 0 ? 0 : 1 + (ft - 1) / R.nt, t = ft == 0 ? 0 : (ft - 1) % R.nt;
    const int jmr = R.jm;
    if (f <= 1) {
        double s = Xc(R, f, i, 1, l, t);
        for (int j = 2; j <= yr; ++j) s = s + Xc(R, f, i, j, l, t);
        Xc(R, f, i, yr, l, t) = s;
        double e = Xc(R, f, i, jmr - yr + 1, l, t);
        for (int j = jmr - yr + 2; j <= jmr; ++j) e = e + Xc(R, f, i, j, l, t);
        Xc(R, f, i, jmr - yr + 1, l, t) = e;
    }
    Xc(R, f, i, yr - 1, l, t) = Xc(R, f, i, 0, l, t);
    Xc(R, f, i, jmr - yr + 2, l, t) = Xc(R, f, i, jmr + 1, l, t);
}

__global__ void k_uncompress_y(RA R, int yr, int is, int ie, int ls, int le, int nfield) {
    int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    const int ni = ie - is + 1, nl = le - ls + 1;
    const int64_t per = (int64_t)ni * nl;
    if (ni <= 0 || nl <= 0 || k >= per * nfield) return;
    const int ft = (int)(k / per), rest = (int)(k % per);
    const int i = is + rest / nl, l = ls + rest % nl;
    const int f = ft == 0 ? 0 : 1 + (ft - 1) / R.nt, t = ft == 0 ? 0 : (ft - 1) % R.nt;
    const int jmr = R.jm;
    const double w = div_ip(Xc(R, f, i, yr, l, t), (double)yr);
    for (int j = 1; j <= yr; ++j) Xc(R, f, i, j, l, t) = w;
    const double e = div_ip(Xc(R, f, i, jmr - yr + 1, l, t), (double)yr);
    for (int j = jmr - yr + 1; j <= jmr; ++j) Xc(R, f, i, j, l, t) = e;
}

// ------------------------------------------------------------------ mix_edges
// One thread per (ring block, level, field, tracer): the block's mean, accumulated rows outer /
// columns inner from 0 over q / (xr yr), spread over the block (exchange.py:178-229).  Ring
// blocks: the first and last block column (when the x edges mix) and the first and last block
// row (children touching no pole), each once, enumerated by ring_block -- only they get threads.
struct Ring {
    int imp, jmp, ncolb, x0, nx, nrow, ysp;
    __host__ __device__ Ring(int imp_, int jmp_, int xedges, int ysp_, int ynp)
        : imp(imp_), jmp(jmp_), ysp(ysp_) {
        ncolb = xedges ? (imp > 1 ? 2 : 1) * jmp : 0;  // the x-edge block columns, all their rows
        x0 = xedges ? 1 : 0;                            // the block columns between them
        nx = (xedges ? imp - 1 : imp) - x0;
        if (nx < 0) nx = 0;
        nrow = (ysp ? 1 : 0) + (ynp && !(ysp && jmp == 1) ? 1 : 0);  // the first and last block rows
    }
    __host__ __device__ int64_t count() const { return ncolb + (int64_t)nrow * nx; }
};
__device__ __forceinline__ void ring_block(const Ring &g, int b, int &ip, int &jp) {
    if (b < g.ncolb) {
        ip = b / g.jmp == 0 ? 0 : g.imp - 1;
        jp = b % g.jmp;
    } else {
        const int b2 = b - g.ncolb, row = b2 / g.nx;
        ip = g.x0 + b2 % g.nx;
        jp = (row == 0 && g.ysp) ? 0 : g.jmp - 1;
    }
}

__global__ void k_mix_edges(RA R, int xr, int yr, Ring g, int nfield) {
    int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    const int64_t per = g.count() * R.lm;
    if (k >= per * nfield) return;
    const int ft = (int)(k / per);
    const int64_t rest = k % per;
    const int b = (int)(rest / R.lm), l = (int)(rest % R.lm) + 1;
    int ip, jp;
    ring_block(g, b, ip, jp);
    const int f = ft == 0 ? 0 : 1 + (ft - 1) / R.nt, t = ft == 0 ? 0 : (ft - 1) % R.nt;
    const double xyref = (double)(xr * yr);
    double acc = 0.0;
    for (int bb = 0; bb < yr; ++bb)
        for (int a = 0; a < xr; ++a) acc = acc + Xc(R, f, ip * xr + a + 1, jp * yr + bb + 1, l, t) / xyref;
    for (int bb = 0; bb < yr; ++bb)
        for (int a = 0; a < xr; ++a) Xc(R, f, ip * xr + a + 1, jp * yr + bb + 1, l, t) = acc;
}

// ------------------------------------------------------------------ update_parent
// One thread per (parent footprint cell, level, field m / rm-tracer): the child's block sum,
// columns outer / rows inner from 0 (exchange.py:233-258).
__global__ void k_update_parent(RA P, RA C, int ib, int jb, int xr, int yr, int nfield) {
    int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    const int imp = C.im / xr, jmp = C.jm / yr;
    const int64_t per = (int64_t)imp * jmp * C.lm;
    if (k >= per * nfield) return;
    const int ft = (int)(k / per);
    const int64_t rest = k % per;
    const int ip = (int)(rest / ((int64_t)jmp * C.lm)), jp = (int)((rest / C.lm) % jmp), l = (int)(rest % C.lm) + 1;
    const int f = ft == 0 ? 0 : 1, t = ft == 0 ? 0 : ft - 1;
    double acc = 0.0;
    for (int a = 0; a < xr; ++a)
        for (int bb = 0; bb < yr; ++bb) acc = acc + Xc(C, f, ip * xr + a + 1, jp * yr + bb + 1, l, t);
    Xc(P, f, ib + ip, jb + jp, l, t) = acc;
}

// ------------------------------------------------------------------ _coarsen_block
// The parent's am, bm, cm and m over the child's footprint rebuilt from the child's
// (massflow.py:334-397).  One thread per (parent face / cell, level, field):
//   field 0  am(ib-1+ip, jb+jp, l) = sum_b am_c(ip xr, jp yr + b + 1, l) tr   (ip = 0..imp)
//   field 1  bm(ib+ip, jb+jp, l)   = sum_a bm_c(ip xr + a + 1, jp yr + 1, l) tr (jp = 0..jmp)
//   field 2  cm(ib+ip, jb+jp, l)   = sum_a sum_b cm_c(., ., l) tr   (l = 1..lm)
//   field 3  m (ib+ip, jb+jp, l)   = sum_b sum_a m_c(., ., l)
__global__ void k_coarsen_block(RA P, RA C, int ib, int jb, int lb, int xr, int yr, double tr) {
    int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    const int imp = C.im / xr, jmp = C.jm / yr, lm = C.lm;
    const int64_t per = (int64_t)(imp + 1) * (jmp + 1) * lm;
    if (k >= per * 4) return;
    const int fld = (int)(k / per);
    const int64_t rest = k % per;
    const int ip = (int)(rest / ((int64_t)(jmp + 1) * lm)), jp = (int)((rest / lm) % (jmp + 1)), l = (int)(rest % lm);
    const int lp = lb + l;  // Fortran level of the parent (l 0-based within the child's 1..lm)
    auto wrap = [&](int i) {  // the parent's i of the child's block column (mod the parent's im)
        int v = (i - 1) % P.im;
        if (v < 0) v += P.im;
        return v + 1;
    };
    if (fld == 0) {
        if (jp >= jmp) return;
        double top = 0.0;
        for (int b = 0; b < yr; ++b) top = top + Fc(C.am, ip * xr, jp * yr + b + 1, l + 1) * tr;
        Fc(P.am, wrap(ib - 1 + ip), jb + jp, lp) = top;
    } else if (fld == 1) {
        if (ip >= imp) return;
        double top = 0.0;
        for (int a = 0; a < xr; ++a) top = top + Fc(C.bm, ip * xr + a + 1, jp * yr + 1, l + 1) * tr;
        Fc(P.bm, wrap(ib + ip), jb + jp, lp) = top;
    } else if (fld == 2) {
        if (ip >= imp || jp >= jmp) return;
        double top = 0.0;
        for (int a = 0; a < xr; ++a)
            for (int b = 0; b < yr; ++b) top = top + Fc(C.cm, ip * xr + a + 1, jp * yr + b + 1, l + 1) * tr;
        Fc(P.cm, wrap(ib + ip), jb + jp, lp) = top;
    } else {
        if (ip >= imp || jp >= jmp) return;
        double top = 0.0;
        for (int b = 0; b < yr; ++b)
            for (int a = 0; a < xr; ++a) top = top + Mc(C, ip * xr + a + 1, jp * yr + b + 1, l + 1);
        Mc(P, wrap(ib + ip), jb + jp, lp) = top;
    }
}

// ------------------------------------------------------------------ coarsen_ambm
// Each child's outer interface fluxes from the parent's face flux divided over the child faces it
// covers (massflow.py:400-428).  One thread per (parent row j / column i, level).
__global__ void k_coarsen_ambm(RA P, RA C, int ib, int ie, int jb, int je, int lb, int le, int xr, int yr, int zr,
                               int xedges, int sp_edge, int np_edge) {
    int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    const int nl = le - lb + 1, nj = je - jb + 1, ni = ie - ib + 1;
    if (k < (int64_t)nj * nl) {
        if (!xedges) return;
        const int j = jb + (int)(k / nl), lev = lb + (int)(k % nl);
        const int jc = (j - jb) * yr + 1, lc = (lev - lb) * zr + 1;
        const double cell1 = div_ip(Fc(P.am, ib - 1, j, lev), (double)(yr * zr));
        const double cellm = div_ip(Fc(P.am, ie, j, lev), (double)(yr * zr));
        for (int jj = jc; jj <= jc + yr - 1; ++jj)
            for (int ll = lc; ll <= lc + zr - 1; ++ll) {
                Fc(C.am, xr - 1, jj, ll) = cell1;
                Fc(C.am, C.im - xr + 1, jj, ll) = cellm;
            }
        return;
    }
    k -= (int64_t)nj * nl;
    if (k >= (int64_t)ni * nl) return;
    const int i = ib + (int)(k / nl), lev = lb + (int)(k % nl);
    const int ic = (i - ib) * xr + 1, lc = (lev - lb) * zr + 1;
    const double cell1 = div_ip(Fc(P.bm, i, jb, lev), (double)(xr * zr));
    const double cellm = div_ip(Fc(P.bm, i, je + 1, lev), (double)(xr * zr));
    for (int ii = ic; ii <= ic + xr - 1; ++ii)
        for (int ll = lc; ll <= lc + zr - 1; ++ll) {
            if (sp_edge) Fc(C.bm, ii, yr, ll) = cell1;
            if (np_edge) Fc(C.bm, ii, C.jm - yr + 2, ll) = cellm;
        }
}

}  // namespace

// views[0..7] of each region: m, rm, rxm, rym, rzm, am, bm, cm (whole arrays)
extern "C" int gb_put_xedges(gb_ctx *ctx, const gb_view *parent, const gb_view *child, int ib, int ie, int jbeg,
                             int lbeg, int xr, int yr, int zr, double yzref, double xyzref, int tracers) {
    RA P = ra(parent), C = ra(child);
    const int nfield = tracers ? 1 + 4 * C.nt : 1;
    const int64_t total = (int64_t)C.jm * C.lm * nfield;
    k_put_xedges<<<grid_for(total), 128, 0, ctx->stream>>>(P, C, ib, ie, jbeg, lbeg, xr, yr, zr, yzref, xyzref, nfield);
    return gb_after_launch(ctx, "put_xedges");
}

extern "C" int gb_put_yedges(gb_ctx *ctx, const gb_view *parent, const gb_view *child, int jb, int je, int ibeg,
                             int lbeg, int xr, int yr, int zr, double xzref, double xyzref, int tracers) {
    RA P = ra(parent), C = ra(child);
    const int nfield = tracers ? 1 + 4 * C.nt : 1;
    const int64_t total = (int64_t)C.im * C.lm * nfield;
    k_put_yedges<<<grid_for(total), 128, 0, ctx->stream>>>(P, C, jb, je, ibeg, lbeg, xr, yr, zr, xzref, xyzref, nfield);
    return gb_after_launch(ctx, "put_yedges");
}

extern "C" int gb_compress_xedges(gb_ctx *ctx, const gb_view *region, int xr, int js, int je, int ls, int le,
                                  int tracers, int uncompress) {
    RA R = ra(region);
    const int nfield = tracers ? 1 + 4 * R.nt : 1;
    const int64_t total = (int64_t)(je - js + 1) * (le - ls + 1) * nfield;
    if (total <= 0) return GB_OK;
    if (uncompress)
        k_uncompress_x<<<grid_for(total), 128, 0, ctx->stream>>>(R, xr, js, je, ls, le, nfield);
    else
        k_compress_x<<<grid_for(total), 128, 0, ctx->stream>>>(R, xr, js, je, ls, le, nfield);
    return gb_after_launch(ctx, "compress_xedges");
}

extern "C" int gb_compress_yedges(gb_ctx *ctx, const gb_view *region, int yr, int is, int ie, int ls, int le,
                                  int tracers, int uncompress) {
    RA R = ra(region);
    const int nfield = tracers ? 1 + 4 * R.nt : 1;
    const int64_t total = (int64_t)(ie - is + 1) * (le - ls + 1) * nfield;
    if (total <= 0) return GB_OK;
    if (uncompress)
        k_uncompress_y<<<grid_for(total), 128, 0, ctx->stream>>>(R, yr, is, ie, ls, le, nfield);
    else
        k_compress_y<<<grid_for(total), 128, 0, ctx->stream>>>(R, yr, is, ie, ls, le, nfield);
    return gb_after_launch(ctx, "compress_yedges");
}

extern "C" int gb_mix_edges(gb_ctx *ctx, const gb_view *region, int xr, int yr, int xedges, int ysp, int ynp,
                            int tracers) {
    RA R = ra(region);
    const int nfield = tracers ? 1 + 4 * R.nt : 1;
    const Ring g(R.im / xr, R.jm / yr, xedges, ysp, ynp);
    const int64_t total = g.count() * R.lm * nfield;
    if (total == 0) return GB_OK;
    k_mix_edges<<<grid_for(total), 128, 0, ctx->stream>>>(R, xr, yr, g, nfield);
    return gb_after_launch(ctx, "mix_edges");
}

extern "C" int gb_update_parent(gb_ctx *ctx, const gb_view *parent, const gb_view *child, int ib, int jb, int xr,
                                int yr, int tracers) {
    RA P = ra(parent), C = ra(child);
    const int nfield = tracers ? 1 + C.nt : 1;
    const int64_t total = (int64_t)(C.im / xr) * (C.jm / yr) * C.lm * nfield;
    k_update_parent<<<grid_for(total), 128, 0, ctx->stream>>>(P, C, ib, jb, xr, yr, nfield);
    return gb_after_launch(ctx, "update_parent");
}

extern "C" int gb_coarsen_block(gb_ctx *ctx, const gb_view *parent, const gb_view *child, int ib, int jb, int lb,
                                int xr, int yr, double tr) {
    RA P = ra(parent), C = ra(child);
    const int64_t total = (int64_t)(C.im / xr + 1) * (C.jm / yr + 1) * C.lm * 4;
    k_coarsen_block<<<grid_for(total), 128, 0, ctx->stream>>>(P, C, ib, jb, lb, xr, yr, tr);
    return gb_after_launch(ctx, "coarsen_block");
}

extern "C" int gb_coarsen_ambm(gb_ctx *ctx, const gb_view *parent, const gb_view *child, int ib, int ie, int jb,
                               int je, int lb, int le, int xr, int yr, int zr, int xedges, int sp_edge,
                               int np_edge) {
    RA P = ra(parent), C = ra(child);
    const int64_t total = (int64_t)((je - jb + 1) + (ie - ib + 1)) * (le - lb + 1);
    k_coarsen_ambm<<<grid_for(total), 128, 0, ctx->stream>>>(P, C, ib, ie, jb, je, lb, le, xr, yr, zr, xedges,
                                                             sp_edge, np_edge);
    return gb_after_launch(ctx, "coarsen_ambm");
}
