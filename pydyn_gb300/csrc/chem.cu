// The CH4 `c` and `s` operators on a region's columns.
//
// k_chem_rows: thread per latitude -- the zonal loss-rate columns' edges (strat_edges), checked
// strictly descending, and the tropopause pressure.  k_chem: thread per (column, level), a warp
// holding one level of 32 columns (cells at one level take the same branches -- above or below
// the tropopause, inside the zonal columns or under them -- so the FP64 pipe issues with its
// lanes full) and a block that warp's neighbouring levels -- the
// cell's half levels and tropospheric Cl edges checked, the four loss rates, decay =
// exp(-(((L1 + L2) + L3) + L4) dt), and either the rates and decay written out (gb_loss_rates,
// every column of the region) or the decay applied to the listed tracers' mass and slopes
// (gb_chemistry, the columns a region owns).  A rebinned layer sums, in input order from +0.0,
// data * thickness over the input layers first .. last-1 whose overlap is positive; the terms
// the reference adds for the others are +0.0, which leave such a sum unchanged.  exp / pow /
// cos are gbmath.h.
//
// k_sources: one thread per owned column: rm(level) += x, rzm(level) -= x.
//
// Reference: pydyn chem.py:59-178 (rebin_many, strat_edges, tropopause, _column, loss_rates,
// decay, apply_decay), zoom/physics.py:55-78 (sources_region, chemistry_region).
#include "gb_common.cuh"
#include "gbmath.h"

namespace {


struct CArgs {
    DV temper, phlb, soil, oh3d, pltrop, cltrop, sp, soh, scl, sod;
    const double *lat, *oh_factor;
    double oh_scale, cl_scale, o1d_scale, soil_rate, dt;
    int im, jm, lm, ns, ntrop, has_trop, has_soil;
    const int32_t *cols;  // (ncol, 2) 0-based (i, j), or null: every column
    int64_t ncol;
    DV loss, decay;             // gb_loss_rates outputs (either may be absent)
    DV q[4];                    // gb_chemistry: rm, rxm, rym, rzm
    uint32_t tracer_mask;       // gb_chemistry: bit t-1 for tracer t
    int apply;
    double *edges, *trop;       // work space: (jm, ns + 1) zonal edges, (jm) tropopause
    DV krates;                  // (im, jm, lm, 2) the rate constants of the temperature, or absent
    double *cache;              // gb_chemistry: CACHE_VALUES per (column, level), or null: value v
                                // of the cell (c, l) at v * ncol * lm + l * ncol + c
    const int32_t *epoch;       // the step counter the cache is keyed by
    gb_ctl *ctl;
};

__device__ __forceinline__ double &E2(const DV &v, int64_t a, int64_t b) { return v.p[a * v.s0 + b * v.s1]; }
__device__ __forceinline__ double &E3(const DV &v, int64_t a, int64_t b, int64_t c) {
    return v.p[a * v.s0 + b * v.s1 + c * v.s2];
}
__device__ __forceinline__ double &E4(const DV &v, int64_t a, int64_t b, int64_t c, int64_t d) {
    return v.p[a * v.s0 + b * v.s1 + c * v.s2 + d * v.s3];
}

// the rate constants of a cell's temperature (chem.py:137-140): OH, 2.45e-12 exp(-1775 / T), and
// tropospheric Cl, (2.36e-12 (T / 298)^1.37) exp(-939 / T)
constexpr double R298 = 1.0 / 298.0;  // correctly rounded: the divisor's reciprocal for div_by_recip
__device__ __forceinline__ double krate_ohf(double T) { return 2.45e-12 * gbm_exp(div_ip(-1775.0, T)); }
__device__ __forceinline__ double krate_cl(double T) {
    return (2.36e-12 * gbm_pow(div_by_recip(T, 298.0, R298), 1.37)) * gbm_exp(div_ip(-939.0, T));
}

// the tropospheric Cl column's edges: pl_trop(i, j, 0 .. ntrop-1), then 0 (chem.py:135)
struct TropEdges {
    const double *p;
    int64_t s;
    int n;
    __device__ double operator[](int k) const { return k < n ? p[k * s] : 0.0; }
};

// The input layers that can overlap the output layer [top, bot] of strictly descending edges
// ip[0..nip] (chem.py:74-75): first = #{k : ip[k+1] >= bot}, last = #{k : ip[k] > top}.  Both
// conditions hold on a prefix of k, so each count is a binary search (the checked order is what
// makes them prefixes; a NaN bound fails every test and counts 0 either way).
template <class Edges>
__device__ void rebin_span(const Edges &ip, int nip, double bot, double top, int &first, int &last) {
    int a = 0, b = nip;
    while (a < b) {
        const int mid = (a + b) >> 1;
        if (gb_ge(ip[mid + 1], bot))
            a = mid + 1;
        else
            b = mid;
    }
    first = a;
    a = 0;
    b = nip;
    while (a < b) {
        const int mid = (a + b) >> 1;
        if (gb_gt(ip[mid], top))
            a = mid + 1;
        else
            b = mid;
    }
    last = a;
}

// rebin_levels(ip_mix) of one output layer [top, bot] from the edges ip[0..nip], its input
// layers first..last-1 (rebin_span)
template <class Edges>
__device__ double rebin_layer(const Edges &ip, int first, int last, const double *data, int64_t stride, double bot,
                              double top) {
    double overlap = 0.0;
    for (int k = first; k < last; ++k) {
        const double thickness = np_min(bot, ip[k]) - np_max(top, ip[k + 1]);
        if (gb_gt0(thickness)) overlap = add_ip(overlap, data[k * stride] * thickness);  // like-signed terms
    }
    const double width = bot - top;
    return gb_gt0(width) ? div_ip(overlap, width) : overlap;
}

// rebin_layer of three columns on the same edges at once (the zonal OH, Cl and O(1D) columns):
// each layer's overlap is made once and added to each column's sum, in input order as before
template <class Edges>
__device__ void rebin_layer3(const Edges &ip, int first, int last, const double *d0, int64_t s0, const double *d1,
                             int64_t s1, const double *d2, int64_t s2, double bot, double top, double &r0, double &r1,
                             double &r2) {
    double o0 = 0.0, o1 = 0.0, o2 = 0.0;
    for (int k = first; k < last; ++k) {
        const double thickness = np_min(bot, ip[k]) - np_max(top, ip[k + 1]);
        if (gb_gt0(thickness)) {
            o0 = add_ip(o0, d0[k * s0] * thickness);  // like-signed terms: the integer pipe's sums
            o1 = add_ip(o1, d1[k * s1] * thickness);
            o2 = add_ip(o2, d2[k * s2] * thickness);
        }
    }
    const double width = bot - top;
    if (gb_gt0(width)) {  // three quotients by one width: its reciprocal, then div_by_recip
        const double y = recip_for(width);
        r0 = div_by_recip(o0, width, y);
        r1 = div_by_recip(o1, width, y);
        r2 = div_by_recip(o2, width, y);
    } else {
        r0 = o0;
        r1 = o1;
        r2 = o2;
    }
}

// thread per (latitude, edge): the zonal columns' edges (strat_edges, chem.py:91-98: midpoints, a
// half layer below the first, 0 above the last, x100), each checked below the one before it (made
// again here by the same statements), and, at edge 0, the tropopause pressure (chem.py:101-104)
__device__ __forceinline__ double strat_edge(const CArgs &A, int j, int k) {
    double e;
    if (k == 0) {
        const double p0 = E2(A.sp, j, 0), p1 = E2(A.sp, j, 1);
        e = p0 + 0.5 * (p0 - p1);
    } else if (k < A.ns) {
        e = (E2(A.sp, j, k - 1) + E2(A.sp, j, k)) / 2.0;
    } else {
        e = 0.0;
    }
    return e * 100.0;
}
__global__ void k_chem_rows(CArgs A) {
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const int ns = A.ns;
    if (t >= (int64_t)A.jm * (ns + 1)) return;
    const int j = (int)(t / (ns + 1)), k = (int)(t % (ns + 1));
    const double e = strat_edge(A, j, k);
    A.edges[(int64_t)j * (ns + 1) + k] = e;
    if (k > 0 && !gb_lt(e, strat_edge(A, j, k - 1)))  // = (edges[k] - edges[k-1] < 0) for every input
        raise_status(A.ctl, GB_ELEVELS);
    if (k == 0) {
        const double cl = gbm_cos(A.lat[j]);
        A.trop[j] = 30000.0 - 21500.0 * (cl * cl);
    }
}

// The cache of gb_chemistry, per (column, level) (value-major, then level, then column: a warp's
// reads are contiguous): the cell's bot and top pressures and the step
// counter it was filled at, then the rates that do not depend on the OH factor -- the zonal OH
// column's rate, L1 (Cl) and L2 (O(1D)) -- and, for a cell above the tropopause (where OH's rate
// is the zonal column's), the decay itself.  A step calls chemistry in pairs on one air mass (the
// end of a half step and the start of the next, nothing in between moves mass): the second call
// of a pair finds the same pressures and step counter and takes these instead of remaking them --
// the same inputs, so the same bits; only the OH factor (the half step's diurnal factor) differs.
constexpr int CACHE_VALUES = 8;

// thread per (column, level): the four rates, the decay, and its use.  Lanes run along the
// columns, warps along the levels: a block is 32 columns at blockDim / 32 consecutive levels.
__global__ void __launch_bounds__(GB_TUNE_MAX_CELL) k_chem(CArgs A) {
    const int lm = A.lm, lv = blockDim.x >> 5;
    const int nlg = (lm + lv - 1) / lv;
    const int64_t c = (int64_t)(blockIdx.x / nlg) * 32 + (threadIdx.x & 31);
    const int l = (int)(blockIdx.x % nlg) * lv + (int)(threadIdx.x >> 5);
    if (c >= A.ncol || l >= lm) return;
    const int64_t ncell = A.ncol * lm, u = (int64_t)l * A.ncol + c;  // u: the cell's place in the cache
    int i, j;
    if (A.cols) {
        i = A.cols[2 * c];
        j = A.cols[2 * c + 1];
    } else {
        i = (int)(c / A.jm);
        j = (int)(c % A.jm);
    }
    const int ns = A.ns, nt = A.ntrop;
    const double *edges = A.edges + (int64_t)j * (ns + 1);
    const double bot = E3(A.phlb, i, j, l), top = E3(A.phlb, i, j, l + 1);
    bool ok = gb_lt(top, bot);  // = (top - bot < 0), exactly: a difference of unequal doubles is never 0
    TropEdges tedges{nullptr, 0, 0};
    if (A.has_trop) {
        tedges = TropEdges{&E3(A.pltrop, i, j, 0), A.pltrop.s2, nt};
        if (l == 0)  // the column's tropospheric edges, checked once
            for (int k = 0; k < nt; ++k) ok = ok && gb_lt(tedges[k + 1], tedges[k]);
    }
    if (!ok) {
        raise_status(A.ctl, GB_ELEVELS);
        return;
    }
    const double trop = A.trop[j];
    const double *doh = &E2(A.soh, j, 0), *dcl = &E2(A.scl, j, 0), *dod = &E2(A.sod, j, 0);

    {
        const bool strat = gb_lt(bot, trop);
        const double T = E3(A.temper, i, j, l);
        double *cc = A.cache ? A.cache + u : nullptr;  // value v at cc[v * ncell]
        const bool hit = cc && __double_as_longlong(cc[0]) == __double_as_longlong(bot) &&
                         __double_as_longlong(cc[ncell]) == __double_as_longlong(top) &&
                         __double_as_longlong(cc[2 * ncell]) == (long long)*A.epoch;
        double s_oh, L1, L2;
        if (hit) {
            s_oh = cc[3 * ncell];
            L1 = cc[4 * ncell];
            L2 = cc[5 * ncell];
        } else {
            const bool below = gb_gt(bot, edges[0]);
            double s_cl = dcl[0], s_od = dod[0];
            s_oh = doh[0];
            if (!below) {  // the three zonal columns share their edges: one overlap search
                int first, last;
                rebin_span(edges, ns, bot, top, first, last);
                rebin_layer3(edges, first, last, doh, A.soh.s1, dcl, A.scl.s1, dod, A.sod.s1, bot, top, s_oh, s_cl,
                             s_od);
            }
            double trop_cl = 0.0;
            if (A.has_trop) {
                const double *dtr = &E3(A.cltrop, i, j, 0);
                double v = dtr[0];
                if (!gb_gt(bot, tedges[0])) {
                    int first, last;
                    rebin_span(tedges, nt, bot, top, first, last);
                    v = rebin_layer(tedges, first, last, dtr, A.cltrop.s2, bot, top);
                }
                const double krate = A.krates.p ? E4(A.krates, i, j, l, 1) : krate_cl(T);
                trop_cl = (v * krate) * A.cl_scale;
            }
            L1 = strat ? s_cl : add_ip(s_cl, trop_cl);  // rates: like-signed sums
            L2 = s_od * A.o1d_scale;
        }
        double L0 = s_oh;
        if (!strat) {  // below the tropopause: OH's own rate, with the half step's factor
            double oh = E3(A.oh3d, i, j, l);
            if (A.oh_factor) oh = oh * A.oh_factor[i];
            const double krate_oh = A.krates.p ? E4(A.krates, i, j, l, 0) : krate_ohf(T);
            L0 = (krate_oh * oh) * A.oh_scale;
        }
        const double L3 = (A.has_soil && l == 0) ? -(A.soil_rate * E2(A.soil, i, j)) : 0.0;
        // the rates are >= 0 and L3 is +0 but at the surface: the sums are the integer pipe's (add_ip;
        // the surface's soil uptake, of the other sign, takes its FP64 fallback)
        const double d = (hit && strat) ? cc[6 * ncell] : gbm_exp(-(add_ip(add_ip(add_ip(L0, L1), L2), L3) * A.dt));
        if (cc && !hit) {
            cc[0] = bot;
            cc[ncell] = top;
            cc[2 * ncell] = __longlong_as_double((long long)*A.epoch);
            cc[3 * ncell] = s_oh;
            cc[4 * ncell] = L1;
            cc[5 * ncell] = L2;
            cc[6 * ncell] = d;  // taken again only above the tropopause, where no input differs
        }
        if (A.apply) {
            for (uint32_t mask = A.tracer_mask; mask; mask &= mask - 1) {
                const int t = __ffs(mask) - 1;
                for (int w = 0; w < 4; ++w) {
                    double &x = E4(A.q[w], i, j, l, t);
                    x = x * d;
                }
            }
        } else {
            if (A.loss.p) {
                E4(A.loss, i, j, l, 0) = L0;
                E4(A.loss, i, j, l, 1) = L1;
                E4(A.loss, i, j, l, 2) = L2;
                E4(A.loss, i, j, l, 3) = L3;
            }
            if (A.decay.p) E3(A.decay, i, j, l) = d;
        }
    }
}

struct SArgs {
    DV rm, rzm, flux;
    const double *area;
    double scale;
    int level, tracer;
    const int32_t *cols;
    int64_t ncol;
};

__global__ void k_sources(SArgs A) {
    const int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= A.ncol) return;
    const int i = A.cols[2 * c], j = A.cols[2 * c + 1];
    double x = E2(A.flux, i, j);
    if (A.area) x = (x * A.area[j]) * A.scale;
    double &rm = E4(A.rm, i, j, A.level, A.tracer);
    double &rz = E4(A.rzm, i, j, A.level, A.tracer);
    rm = rm + x;
    rz = rz - x;
}

int setup_chem(CArgs &A, const gb_view *temper, const gb_view *phlb, const double *lat, const gb_view *strat_press,
               const gb_view *strat_oh, const gb_view *strat_cl, const gb_view *strat_od, const gb_view *oh_3d,
               const gb_view *pl_trop, const gb_view *cl_trop, const gb_view *soil, const double *oh_factor,
               double oh_scale, double cl_scale, double o1d_scale, double soil_rate, double dt) {
    if (!temper || !phlb || !lat || !strat_press || !strat_oh || !strat_cl || !strat_od || !oh_3d) return GB_EARG;
    if ((pl_trop == nullptr) != (cl_trop == nullptr)) {
        gb_set_error("chemistry: pl_trop and cl_trop go together");
        return GB_EARG;
    }
    A.temper = dv(temper); A.phlb = dv(phlb); A.oh3d = dv(oh_3d);
    A.sp = dv(strat_press); A.soh = dv(strat_oh); A.scl = dv(strat_cl); A.sod = dv(strat_od);
    A.im = (int)temper->n[0]; A.jm = (int)temper->n[1]; A.lm = (int)temper->n[2];
    A.ns = (int)strat_press->n[1];
    if (A.ns < 2 || phlb->n[2] != A.lm + 1) {
        gb_set_error("chemistry: need >= 2 zonal levels and phlb of lm+1 half levels");
        return GB_EARG;
    }
    A.has_trop = pl_trop != nullptr;
    if (A.has_trop) {
        A.pltrop = dv(pl_trop); A.cltrop = dv(cl_trop);
        A.ntrop = (int)pl_trop->n[2];
    }
    A.has_soil = soil != nullptr;
    if (A.has_soil) A.soil = dv(soil);
    A.lat = lat; A.oh_factor = oh_factor;
    A.oh_scale = oh_scale; A.cl_scale = cl_scale; A.o1d_scale = o1d_scale; A.soil_rate = soil_rate; A.dt = dt;
    return GB_OK;
}

int launch_chem(gb_ctx *ctx, CArgs &A) {
    A.ctl = ctx->ctl;
    if (A.ncol == 0) return GB_OK;
    double *w = gb_work(ctx, (size_t)A.jm * (A.ns + 2) * sizeof(double));
    if (!w) return GB_ECUDA;
    A.edges = w;
    A.trop = w + (size_t)A.jm * (A.ns + 1);
    k_chem_rows<<<(unsigned)(((int64_t)A.jm * (A.ns + 1) + 127) / 128), 128, 0, ctx->stream>>>(A);
    if (int rc = gb_after_launch(ctx, "chem_rows")) return rc;
    // blocks of 32 columns x (tcell / 32) levels
    const int tcell = ctx->tune[GB_TUNE_CELL_THREADS], lv = tcell / 32;
    const int64_t blocks = (A.ncol + 31) / 32 * ((A.lm + lv - 1) / lv);
    k_chem<<<(unsigned)blocks, tcell, 0, ctx->stream>>>(A);
    return gb_after_launch(ctx, A.apply ? "chemistry" : "loss_rates");
}

}  // namespace

extern "C" int gb_loss_rates(gb_ctx *ctx, const gb_view *temper, const gb_view *phlb, const double *lat,
                             const gb_view *strat_press, const gb_view *strat_oh, const gb_view *strat_cl,
                             const gb_view *strat_od, const gb_view *oh_3d, const gb_view *pl_trop,
                             const gb_view *cl_trop, const gb_view *soil, const double *oh_factor, double oh_scale,
                             double cl_scale, double o1d_scale, double soil_rate, double dt_sec,
                             const gb_view *loss, const gb_view *decay) {
    if (!ctx) return GB_EARG;
    CArgs A{};
    if (int rc = setup_chem(A, temper, phlb, lat, strat_press, strat_oh, strat_cl, strat_od, oh_3d, pl_trop, cl_trop,
                            soil, oh_factor, oh_scale, cl_scale, o1d_scale, soil_rate, dt_sec))
        return rc;
    A.loss = loss ? dv(loss) : DV{};
    A.decay = decay ? dv(decay) : DV{};
    A.ncol = (int64_t)A.im * A.jm;
    return launch_chem(ctx, A);
}

extern "C" int gb_chemistry(gb_ctx *ctx, const gb_view *temper, const gb_view *phlb, const double *lat,
                            const gb_view *strat_press, const gb_view *strat_oh, const gb_view *strat_cl,
                            const gb_view *strat_od, const gb_view *oh_3d, const gb_view *pl_trop,
                            const gb_view *cl_trop, const gb_view *soil, const double *oh_factor, double oh_scale,
                            double cl_scale, double o1d_scale, double soil_rate, double dt_sec, const int32_t *cols,
                            int ncol, uint32_t tracer_mask, const gb_view *rm, const gb_view *rxm,
                            const gb_view *rym, const gb_view *rzm, const gb_view *krates, double *cache,
                            const int32_t *epoch) {
    if (!ctx || !rm || !rxm || !rym || !rzm || (ncol > 0 && !cols) || ncol < 0) return GB_EARG;
    if (cache && !epoch) return GB_EARG;
    CArgs A{};
    if (int rc = setup_chem(A, temper, phlb, lat, strat_press, strat_oh, strat_cl, strat_od, oh_3d, pl_trop, cl_trop,
                            soil, oh_factor, oh_scale, cl_scale, o1d_scale, soil_rate, dt_sec))
        return rc;
    A.krates = krates ? dv(krates) : DV{};
    if (rm->n[3] < 32 && (tracer_mask >> rm->n[3]) != 0) {
        gb_set_error("gb_chemistry: a tracer of the mask is beyond the arrays' nt");
        return GB_EARG;
    }
    A.q[0] = dv(rm); A.q[1] = dv(rxm); A.q[2] = dv(rym); A.q[3] = dv(rzm);
    A.cache = cache;
    A.epoch = epoch;
    A.tracer_mask = tracer_mask;
    A.apply = 1;
    A.cols = cols;
    A.ncol = ncol;
    return launch_chem(ctx, A);
}

namespace {
__global__ void k_chem_krates(DV temper, DV krates, const int32_t *cols, int64_t ncol, int jm, int lm) {
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= ncol * lm) return;
    const int64_t c = t / lm;
    const int l = (int)(t % lm);
    const int i = cols ? cols[2 * c] : (int)(c / jm), j = cols ? cols[2 * c + 1] : (int)(c % jm);
    const double T = E3(temper, i, j, l);
    E4(krates, i, j, l, 0) = krate_ohf(T);
    E4(krates, i, j, l, 1) = krate_cl(T);
}
}  // namespace

extern "C" int gb_chem_krates(gb_ctx *ctx, const gb_view *temper, const int32_t *cols, int ncol,
                              const gb_view *krates) {
    if (!ctx || !temper || !krates || ncol < 0) return GB_EARG;
    if (krates->n[0] != temper->n[0] || krates->n[1] != temper->n[1] || krates->n[2] != temper->n[2] ||
        krates->n[3] != 2) {
        gb_set_error("gb_chem_krates: krates must be (im, jm, lm, 2) over temper's (im, jm, lm)");
        return GB_EARG;
    }
    const int64_t n = cols ? (int64_t)ncol : temper->n[0] * temper->n[1];
    const int lm = (int)temper->n[2];
    if (n == 0) return GB_OK;
    const int tcell = ctx->tune[GB_TUNE_CELL_THREADS];
    k_chem_krates<<<gb_blocks(n * lm, tcell), tcell, 0, ctx->stream>>>(
        dv(temper), dv(krates), cols, n, (int)temper->n[1], lm);
    return gb_after_launch(ctx, "chem_krates");
}

extern "C" int gb_sources(gb_ctx *ctx, const gb_view *rm, const gb_view *rzm, const gb_view *flux,
                          const double *area, double scale, int level, int tracer, const int32_t *cols, int ncol) {
    if (!ctx || !rm || !rzm || !flux || (ncol > 0 && !cols) || ncol < 0) return GB_EARG;
    if (level < 1 || level > rm->n[2] || tracer < 1 || tracer > rm->n[3]) {
        gb_set_error("gb_sources: level or tracer (1-based) outside the arrays");
        return GB_EARG;
    }
    if (ncol == 0) return GB_OK;
    SArgs A{};
    A.rm = dv(rm); A.rzm = dv(rzm); A.flux = dv(flux);
    A.area = area; A.scale = scale;
    A.level = level - 1; A.tracer = tracer - 1;
    A.cols = cols; A.ncol = ncol;
    k_sources<<<(unsigned)((ncol + 127) / 128), 128, 0, ctx->stream>>>(A);
    return gb_after_launch(ctx, "sources");
}
