/*
 * gbdyn.h -- C ABI of the GB300 (sm_103a) float64 dynamic step of TM5 as pydyn transcribes it.
 *
 * Every entry point returns GB_OK (0) or a status code; gb_last_error() gives the message of
 * the last failure on the calling thread.  Arrays are device memory described by gb_view:
 * a pointer plus up to four extents and element strides (the layout of a NumPy view of a
 * C-contiguous pydyn array, any strides).  Work is enqueued on the context's one stream and
 * returns without waiting; errors found on the device (a sub-cycle cap reached, non-zero halo
 * faces, a search that would not converge) land in a device status word that gb_sync() reads.
 *
 * The reference interface each entry point replaces is named beside it, by file:line inside
 * the pydyn project (pydyn/kernels.py, pydyn/zoom/..., pydyn/cfl.py, pydyn/diffusion.py,
 * pydyn/chem.py); the device port of pydyn (pydyn/gpu/kernels.py) had the same roles.
 */
#ifndef GBDYN_H
#define GBDYN_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* status codes (bit flags in the device status word) */
enum {
    GB_OK = 0,
    GB_ECFL = 1,      /* a sub-cycle cap was reached: pydyn.kernels.CFLError (kernels.py:60) */
    GB_EHALO = 2,     /* non-zero polar / boundary faces: the ValueError of kernels.py:233,301 */
    GB_ELEVELS = 4,   /* rebin levels not strictly descending: chem.py:47-49 */
    GB_ESEARCH = 8,   /* a region-wide sub-cycle search did not settle in its rounds */
    GB_EARG = 16,     /* bad argument (host side) */
    GB_ECUDA = 32,    /* a CUDA runtime call failed */
    GB_ETIMEOUT = 64  /* a bounded device wait ran out */
};

typedef struct gb_ctx gb_ctx;

/* A strided float64 (or int32) device array of rank <= 4; unused axes have n = 1, s = 0. */
typedef struct {
    void *p;
    int64_t n[4];
    int64_t s[4]; /* element strides */
} gb_view;

/* ------------------------------------------------------------------ context, memory, stream */
int gb_create(int device, gb_ctx **out);
void gb_destroy(gb_ctx *ctx);
const char *gb_last_error(void);
int gb_alloc(gb_ctx *ctx, size_t bytes, void **dptr);
int gb_free(gb_ctx *ctx, void *dptr);
int gb_put(gb_ctx *ctx, void *dst, const void *src, size_t bytes);      /* host -> device, async */
int gb_get(gb_ctx *ctx, void *dst, const void *src, size_t bytes);      /* device -> host, waits */
int gb_get_async(gb_ctx *ctx, void *dst, const void *src, size_t bytes); /* device -> pinned host */
int gb_copy_d2d(gb_ctx *ctx, void *dst, const void *src, size_t bytes); /* async */
int gb_host_alloc(size_t bytes, void **hptr);                           /* pinned host memory */
int gb_host_free(void *hptr);
int gb_stream_sync(gb_ctx *ctx);   /* wait for the stream */
int gb_sync(gb_ctx *ctx);          /* wait for the stream, then read and clear the status word */
int gb_status_peek(gb_ctx *ctx, int *word); /* read the status word without clearing it */
int64_t gb_launches(gb_ctx *ctx);  /* kernels this context has launched (graph replays count theirs) */
void *gb_stream(gb_ctx *ctx);      /* the cudaStream_t work is enqueued on */

/* CUDA graphs of enqueued work: a whole step is captured once and replayed. */
int gb_capture_begin(gb_ctx *ctx);
int gb_capture_end(gb_ctx *ctx, void **graph);
int gb_graph_launch(gb_ctx *ctx, void *graph);
int gb_graph_destroy(void *graph);

/* Launch shapes the autotuner sets per context (pydyn_gb300.tune).  They choose how work is
 * laid onto threads and blocks, never what any element computes: results are bitwise the same
 * for every accepted value.  No reference counterpart (pydyn has no device launch shapes). */
#define GB_TUNE_COLUMN_THREADS 0 /* thread-per-column kernels (convection chains, Kzz columns): 32..256 */
#define GB_TUNE_CELL_THREADS 1   /* thread-per-cell kernels (convection matrix, Kzz, chemistry): 32..512 */
#define GB_TUNE_LU_WARPS 2       /* columns (one warp each) per block of the convection LU: 1, 2, 4 */
#define GB_TUNE_APPLY_THREADS 3  /* the convection apply's smallest block (whole columns): 32..1024;
                                   0 (the default): the columns a block that even out the FP64
                                   work over the SMs */
#define GB_TUNE_LU_LANES 4       /* lanes per column of the convection LU (32 / lanes columns a warp): 8, 16, 32 */
#define GB_TUNE_N 5
int gb_device_name(gb_ctx *ctx, char *buf, int len); /* "<name> sm_<cc> x<SMs>": the tuning cache's key */
/* The context's work space (what operators allocate lazily outside a capture): at least bytes
 * from now on, and its present size -- a context that will run captured work first takes the
 * size another context's uncaptured run grew to. */
int gb_work_reserve(gb_ctx *ctx, size_t bytes);
/* The context's streams at `rank` steps above the device's least priority (0: the default,
 * clamped to the greatest): the block scheduler serves a higher stream's kernels first.  A
 * captured graph keeps each kernel at the priority of the stream it was captured on.  Waits for
 * the context's work; not while capturing. */
int gb_stream_priority(gb_ctx *ctx, int rank);
size_t gb_work_size(gb_ctx *ctx);
/* The context's int32 scratch (the sub-cycle searches' counts and candidates): its device
 * address and length in elements, for diagnostics and tests.  No reference counterpart. */
int gb_scratch_info(gb_ctx *ctx, int32_t **ptr, size_t *n);
int gb_tune_set(gb_ctx *ctx, int key, int value); /* GB_EARG for a value outside the key's range */
int gb_tune_get(gb_ctx *ctx, int key, int *value);

/* Timing: events recorded on the context's stream. */
int gb_event_create(void **ev);
int gb_event_record(gb_ctx *ctx, void *ev);
/* Work enqueued on the context's stream after this call waits for the event (recorded on
 * another context's stream): how an ensemble bounds how many members run at once. */
int gb_stream_wait(gb_ctx *ctx, void *ev);
int gb_event_elapsed_ms(void *start, void *stop, float *ms);
/* The host waits until the work before the event's last record has completed (a host pipeline's
 * wait for one step's result while the next runs). */
int gb_event_sync(void *ev);
int gb_event_destroy(void *ev);

/* The Check_CFL rehearsal flag: the mass-only kernels set it on a failed operator, and every
 * later rehearsal kernel returns without work while it is set (advectm_cfl's early return,
 * zoom/check_cfl.py:222-236). */
int gb_cfl_reset(gb_ctx *ctx);
int gb_cfl_failed(gb_ctx *ctx, int *failed); /* waits for the stream */

/* ------------------------------------------------------------------ box statements
 * Elementwise statements on views of equal extents (dst may alias a source exactly).
 * op: 0 dst = a; 1 dst = a * x; 2 dst = a / x; 3 dst = x (fill); 4 dst = a + b; 5 dst = a - b;
 *     6 dst = a * b; 7 dst = a / b; 8 dst = (a * x) / y (the progressive rescale, ops.py:304);
 *     9 dst = x * a + y * b (time interpolation, balance.py:63); 10 dst = x * a (scalar first)
 * These carry the exchange, save/restore and halo statements of pydyn/zoom (exchange.py,
 * host.py:56-70); evaluation per element is the NumPy statement's. */
int gb_box(gb_ctx *ctx, int op, const gb_view *dst, const gb_view *a, const gb_view *b, double x,
           double y);
/* dst = w[0] a + w[1] b, the weights read from device memory when the kernel runs, so that a
 * captured step replays with each step's weights (balance.py:63 time_interpolation). */
int gb_interp(gb_ctx *ctx, const gb_view *dst, const gb_view *a, const gb_view *b, const double *w);
/* counter[0] += delta on the stream (device int32): a step counter that a captured step
 * advances each time it replays (convection's inverse cache epoch). */
int gb_iadd(gb_ctx *ctx, int32_t *counter, int delta);
/* buf[slot] = the GPU's global nanosecond timer when the stream reaches this point (a one-thread
 * kernel, capturable): the timeline of a captured interval's streams
 * (python -m pydyn_gb300.profile --timeline).  No reference counterpart. */
int gb_stamp(gb_ctx *ctx, uint64_t *buf, int slot);
/* n device-to-device copies in one launch: `table` (device memory, 3n uint64) holds each copy's
 * destination, source and byte count (a multiple of 8, each at most max_bytes, the ranges
 * disjoint): a captured interval's first copies (its speculation backup) in one node instead of
 * one each.  No reference counterpart. */
int gb_copy_many(gb_ctx *ctx, const uint64_t *table, int n, size_t max_bytes);
/* dst = seqsum of src over `axis` (src's extent along it), accumulated in index order
 * (ops.seqsum, ops.py:235); dst has src's extents with that axis dropped (n = 1). */
int gb_seqsum(gb_ctx *ctx, const gb_view *dst, const gb_view *src, int axis, double post_mul);

/* ------------------------------------------------------------------ Meteo_Setup_Mass (pydyn/balance.py, zoom_meteo.py)
 * pydyn's layout without halos: pu (im+1, jm, lm), pv (im, jm+1, lm), pw (im, jm, lm+1), dm_dt
 * and the residual (im, jm, lm), sp (im, jm); levi_db (lm) and area (jm) are device float64.
 * dm_dt = ((|levi_db| (sp2 - sp1) / g) area) / dt (balance.py:76-82). */
int gb_fill_mass_change(gb_ctx *ctx, const gb_view *dm_dt, const gb_view *sp1, const gb_view *sp2,
                        const double *levi_db, const double *area, double dt_sec);
/* CheckMassBalance (balance.py:85-94): out (device, 2 float64) = the rms and the largest
 * |diff| of the column convergence's relative mismatch with the pressure tendency (the rms
 * summed in a fixed tree order, not NumPy's). */
int gb_mass_check(gb_ctx *ctx, const gb_view *pu, const gb_view *pv, const gb_view *sp1,
                  const gb_view *sp2, const double *area, double dt_sec, double *out);
/* One BalanceMassFluxes_m of a doubly periodic region (balance.py:107-124, 183-199): every
 * level's residual divergence solved by the periodic Poisson equation -- a float64 discrete
 * Fourier transform (tw_i, tw_j: cos and sin of 2 pi t / N, 2N each; fac (im, jm) the
 * Laplacian's eigenvalues, fac(0, 0) = 1) -- and its gradient added to pu, pv. */
int gb_balance_fft(gb_ctx *ctx, const gb_view *pu, const gb_view *pv, const gb_view *pw,
                   const gb_view *dm_dt, const double *tw_i, const double *tw_j, const double *fac);
/* Match 'sum' of a child to its parent (zoom_meteo.py:87-119): kind 0 the x faces, 1 the y
 * faces, 2 the cells; ri, rj the refinement, ci1..ci2, cj1..cj2 the parent cells covered
 * (1-based); every level; the child in place. */
int gb_match_sum(gb_ctx *ctx, int kind, const gb_view *parent, const gb_view *child, int ri, int rj,
                 int ci1, int ci2, int cj1, int cj2);
/* One BalanceMassFluxes_m of a child against its parent (zoom_meteo.py:163-181): the residual
 * of every level, then per parent cell (cj outer, ci inner) its block's residual through the
 * direct matrices m_to_u (n x (ri+1) rj), m_to_v (n x ri (rj+1)) -- row k the correction of
 * the unit divergence at cell k, n = ri rj <= 64 -- added to the block's faces. */
int gb_balance_direct(gb_ctx *ctx, const gb_view *pu, const gb_view *pv, const gb_view *pw,
                      const gb_view *dm_dt, const double *m_to_u, const double *m_to_v, int ri, int rj,
                      int ci1, int ci2, int cj1, int cj2);

/* ------------------------------------------------------------------ the replay of a dump set
 * (pydyn/replay.py, gpu/engine.py)
 * The engine's comparison of a state array with a dump's (DeviceEngine.compare and .report,
 * which pydyn's engine makes on the host after downloading the state array; replay.py:277-289,
 * harness.py:140-179): a and b of one extent, any strides.  out, a device buffer of 5 int64,
 * receives the number of elements whose bit patterns differ, the largest ulp distance, the bit
 * patterns of the largest |a - b| and of the largest |a - b| / max(|a|, |b|) over the differing
 * elements (NaN propagating), and the first differing element's row-major index (INT64_MAX when
 * none differs).  Stream-ordered. */
int gb_compare(gb_ctx *ctx, const gb_view *a, const gb_view *b, long long *out);

/* ------------------------------------------------------------------ advection (pydyn/kernels.py)
 * x: dynamu on every (j, l) row of a region (kernels.py:129-220, redgrid.py:56-110,
 * zoom/advect.py:237-275).  m (im, jm, lm), tracers (im, jm, lm, nt) sharing strides,
 * am (im+1, jm, lm).  clust (jm) int32 device array: the reduced-grid cluster size of each
 * latitude (1 = uniform), or NULL.  halo: 1 also writes the periodic halos m/rm..(0, j) and
 * (im+1, j) as zoom/advect.py:257-272 does (the views must then sit inside halo'd arrays).
 * nloop_out (jm*lm int32) / amax_out (jm*lm float64): optional device outputs per row. */
int gb_advect_x(gb_ctx *ctx, const gb_view *m, const gb_view *rm, const gb_view *rxm,
                const gb_view *rym, const gb_view *rzm, const gb_view *am, const int32_t *clust,
                int halo, int js, int je, int limits, int max_nloop, int32_t *nloop_out,
                double *amax_out);
/* y: dynamv (kernels.py:223-291 + zoom/advect.py:201-226).  m (im, jm, lm), bm (im, jm+1, lm);
 * bm_full: the whole halo'd bm whose every face of each layer is rescaled with it (or NULL);
 * bm_full_l0: the level of bm_full that is bm's level 0.  nloop_out: lm int32 (optional). */
int gb_advect_y(gb_ctx *ctx, const gb_view *m, const gb_view *rm, const gb_view *rxm,
                const gb_view *rym, const gb_view *rzm, const gb_view *bm, const gb_view *bm_full,
                int bm_full_l0, int limits, int max_nloop, int32_t *nloop_out);
/* gb_advect_y without an allocation.  No counterpart in the reference.  The same arguments and
 * results as gb_advect_y; its per-layer sub-cycle counts are kept in a fixed device array of
 * GB_NOALLOC_MAX_LEVELS int32 (4 KiB) compiled into the library, not in the context's scratch.
 * For callers that must not allocate device memory while they run: a host whose own allocator
 * has reserved the device's free memory, or a loop that cannot take the device-wide
 * synchronisation an allocation may cause.  The call allocates nothing (no cudaMalloc, no
 * library that allocates).  More than GB_NOALLOC_MAX_LEVELS levels return GB_EARG.  Nothing in
 * the array must start at zero: each call writes every count it reads.  The array is one per
 * device, shared by every context and stream: calls that can overlap (two streams, two host
 * threads) race on it and must be serialised by the caller.  The first call on a device looks
 * the array's address up (cudaGetSymbolAddress); make it before any stream capture begins.
 * The looked-up address is kept for the life of the process: after a cudaDeviceReset the
 * library's module is loaded anew and the array may move, so the entry point must not be
 * called again in that process.  The current device must be the context's. */
#define GB_NOALLOC_MAX_LEVELS 1024
int gb_advect_y_noalloc(gb_ctx *ctx, const gb_view *m, const gb_view *rm, const gb_view *rxm,
                        const gb_view *rym, const gb_view *rzm, const gb_view *bm,
                        const gb_view *bm_full, int bm_full_l0, int limits, int max_nloop,
                        int32_t *nloop_out);
/* z: dynamw (kernels.py:295-346).  cm (im, jm, lm+1); cm is left bitwise as it was.
 * n_out: 1 int32 (optional). */
int gb_advect_z(gb_ctx *ctx, const gb_view *m, const gb_view *rm, const gb_view *rxm,
                const gb_view *rym, const gb_view *rzm, const gb_view *cm, int limits,
                int iter_limit, int32_t *n_out);

/* z on a scope: the search looks at every column of m (im, jm, lm), the sub-steps run on the
 * columns [si0, si1) x [sj0, sj1) (0-based, half-open) -- a child's dynamw
 * (zoom/advect.py:444-472, column_trial :415-441). */
int gb_advect_z_scope(gb_ctx *ctx, const gb_view *m, const gb_view *rm, const gb_view *rxm,
                      const gb_view *rym, const gb_view *rzm, const gb_view *cm, int si0, int si1,
                      int sj0, int sj1, int limits, int iter_limit);

/* A child's held-end rows: m (n, nj, nl) cells is-1..ie+1 whose two ends are held, am (n-1, nj,
 * nl) the interior faces (zoom/advect.py:278-345 _dynamu_child, _rows_child, _substeps_child). */
int gb_advect_x_held(gb_ctx *ctx, const gb_view *m, const gb_view *rm, const gb_view *rxm,
                     const gb_view *rym, const gb_view *rzm, const gb_view *am, int limits,
                     int max_nloop);
/* A child's held-end columns: m (ni, n, nl), bm (ni, n-1, nl); bm_full the whole halo'd bm,
 * own[4] (int32, host memory) the inclusive (i0, i1, j0, j1) box of its faces the columns own
 * (zoom/advect.py:348-412 _dynamv_child). */
int gb_advect_y_held(gb_ctx *ctx, const gb_view *m, const gb_view *rm, const gb_view *rxm,
                     const gb_view *rym, const gb_view *rzm, const gb_view *bm, const gb_view *bm_full,
                     int bm_full_l0, const int32_t *own, int limits, int max_nloop);

/* ------------------------------------------------------------------ Check_CFL mass kernels (pydyn/cfl.py)
 * dynamum (cfl.py:140) with the region-1 halos of zoom/check_cfl.py:94-110 when halo = 1. */
int gb_cfl_x(gb_ctx *ctx, const gb_view *m, const gb_view *am, const int32_t *clust, int halo,
             int js, int je, int max_nloop);
/* dynamvm (cfl.py:170) */
int gb_cfl_y(gb_ctx *ctx, const gb_view *m, const gb_view *bm, int max_nloop);
/* dynamwm / zoom _dynamwm (cfl.py:186, zoom/check_cfl.py:206-216): the Courant search over the
 * whole m (im, jm, lm) under cm (im, jm, lm+1), the mass advanced on the scope
 * [si0, si1) x [sj0, sj1) (0-based, half-open) when every column passes. */
int gb_cfl_z(gb_ctx *ctx, const gb_view *m, const gb_view *cm, int si0, int si1, int sj0, int sj1,
             int iter_limit);

/* a child's dynamum / dynamvm (zoom/check_cfl.py:113-193) on held rows / columns */
int gb_cfl_x_held(gb_ctx *ctx, const gb_view *m, const gb_view *am, int max_nloop);
int gb_cfl_y_held(gb_ctx *ctx, const gb_view *m, const gb_view *bm, const gb_view *bm_full,
                  int bm_full_l0, const int32_t *own, int max_nloop);

/* ------------------------------------------------------------------ the zoom exchange
 * Region arguments are arrays of eight gb_views of the whole (halo'd) arrays m, rm, rxm, rym,
 * rzm, am, bm, cm; indices are Fortran (pydyn zoom/exchange.py, zoom/massflow.py). */
/* put_xedges / putm_xedges (exchange.py:17-60) */
int gb_put_xedges(gb_ctx *ctx, const gb_view *parent, const gb_view *child, int ib, int ie, int jbeg,
                  int lbeg, int xr, int yr, int zr, double yzref, double xyzref, int tracers);
/* put_yedges / putm_yedges (exchange.py:63-105) */
int gb_put_yedges(gb_ctx *ctx, const gb_view *parent, const gb_view *child, int jb, int je, int ibeg,
                  int lbeg, int xr, int yr, int zr, double xzref, double xyzref, int tracers);
/* _compress_xedges / _uncompress_xedges (exchange.py:108-141) on rows js..je, levels ls..le */
int gb_compress_xedges(gb_ctx *ctx, const gb_view *region, int xr, int js, int je, int ls, int le,
                       int tracers, int uncompress);
/* _compress_yedges / _uncompress_yedges (exchange.py:144-175) on columns is..ie */
int gb_compress_yedges(gb_ctx *ctx, const gb_view *region, int yr, int is, int ie, int ls, int le,
                       int tracers, int uncompress);
/* mix_edges / mixm_edges (exchange.py:178-229) */
int gb_mix_edges(gb_ctx *ctx, const gb_view *region, int xr, int yr, int xedges, int ysp, int ynp,
                 int tracers);
/* update_parent / updatem_parent (exchange.py:233-258) */
int gb_update_parent(gb_ctx *ctx, const gb_view *parent, const gb_view *child, int ib, int jb, int xr,
                     int yr, int tracers);
/* _coarsen_block (zoom/massflow.py:334-397) */
int gb_coarsen_block(gb_ctx *ctx, const gb_view *parent, const gb_view *child, int ib, int jb, int lb,
                     int xr, int yr, double tr);
/* coarsen_ambm (zoom/massflow.py:400-428) */
int gb_coarsen_ambm(gb_ctx *ctx, const gb_view *parent, const gb_view *child, int ib, int ie, int jb,
                    int je, int lb, int le, int xr, int yr, int zr, int xedges, int sp_edge,
                    int np_edge);

/* ------------------------------------------------------------------ convection (pydyn/kernels.py)
 * convec on the listed owned columns (kernels.py:350-457, zoom/physics.py:33-52): m and tracers
 * the region's interior views (im, jm, lm[, nt]); entu, detu, entd, detd (im, jm, >= lmax);
 * dkg (im, jm, >= lmax); cloud_top / cloud_lfs (im, jm) int32 device arrays with element
 * strides ts0, ts1 (1-based levels, 0 = no cloud); cols: ncol (i, j) int32 pairs, 0-based;
 * dt = nconv / (2 tref).  cache_inv (ncol*lmax*lmax), cache_m (ncol*lmax), cache_tag (ncol)
 * and epoch (1 int32, all device) keep each column's inverse for the next call in the same
 * epoch whose air mass is bitwise unchanged; NULL cache_inv disables the reuse. */
int gb_convec(gb_ctx *ctx, const gb_view *m, const gb_view *rm, const gb_view *rxm, const gb_view *rym,
              const gb_view *rzm, const gb_view *entu, const gb_view *detu, const gb_view *entd,
              const gb_view *detd, const gb_view *dkg, const int32_t *cloud_top,
              const int32_t *cloud_lfs, int64_t ts0, int64_t ts1, const int32_t *cols, int ncol,
              double dt, int lmax, double *cache_inv, double *cache_m, int32_t *cache_tag,
              const int32_t *epoch);

/* Calc_Kzz (diffusion.py:266-276, the zoom driver's Kzz body at zoom/driver.py:186-200): the
 * vertical diffusion exchange rate dkg (im, jm, lmax_conv) of every column, zero at lmax_conv-1.
 * spm, sp (im, jm) the surface pressure of the previous / current instant; pu (im+1, jm, lm),
 * pv (im, jm+1, lm); t, q (im, jm, lm); surface: 10 (im, jm) views in the order oro, lsm, sr,
 * srols, u10m, v10m, sshf, slhf, ewss, nsss; at, bt (lm+1), dxyp (jm) device; dx, dy, ybeg the
 * region's grid in degrees.  pblh (im, jm) receives the boundary-layer height if not NULL. */
int gb_calc_kzz(gb_ctx *ctx, const gb_view *spm, const gb_view *sp, const gb_view *pu,
                const gb_view *pv, const gb_view *t, const gb_view *q, const gb_view *surface,
                const double *at, const double *bt, const double *dxyp, int lmax_conv, double dx,
                double dy, double ybeg, const gb_view *dkg, const gb_view *pblh);

/* CH4 loss rates and decay (chem.py:114-170, loss_rates + decay) of every column of a region:
 * temper, oh_3d (im, jm, lm); phlb (im, jm, lm+1) half levels; lat (jm) radians, device;
 * strat_press (hPa), strat_oh, strat_cl, strat_od (jm, ns >= 2) zonal columns; pl_trop, cl_trop
 * (im, jm, ntrop) the tropospheric Cl column (both NULL: not applied); soil (im, jm) or NULL;
 * oh_factor (im) device, a per-longitude multiplier of oh_3d, or NULL.  Outputs loss
 * (im, jm, lm, 4) and decay (im, jm, lm) = exp(-(sum of the rates) dt_sec), either NULL.
 * Levels that are not strictly descending raise GB_ELEVELS (chem.py:47-49). */
int gb_loss_rates(gb_ctx *ctx, const gb_view *temper, const gb_view *phlb, const double *lat,
                  const gb_view *strat_press, const gb_view *strat_oh, const gb_view *strat_cl,
                  const gb_view *strat_od, const gb_view *oh_3d, const gb_view *pl_trop,
                  const gb_view *cl_trop, const gb_view *soil, const double *oh_factor,
                  double oh_scale, double cl_scale, double o1d_scale, double soil_rate,
                  double dt_sec, const gb_view *loss, const gb_view *decay);
/* chemistry_region (zoom/physics.py:67-78 with chem.loss_rates, decay, apply_decay): the same
 * inputs; on the listed columns cols (ncol, 2) int32 0-based (i, j), device, rm, rxm, rym, rzm
 * (im, jm, lm, nt) of every tracer t whose bit t-1 is set in tracer_mask are multiplied by the
 * cell's decay.  The other columns are left as they are (the reference's factor 1.0).  krates:
 * the rate constants of temper made by gb_chem_krates (the same values), or NULL.  cache: NULL,
 * or 8 doubles per (listed column, level) kept between calls, with epoch (a device int32 step
 * counter, changed whenever temper, the rate constants or dt may change): a call that finds a
 * cell's bot and top pressures and the counter as the last call left them takes the rates that
 * do not depend on oh_factor from there (and, above the tropopause, the decay) -- the same values
 * it would compute.  No reference counterpart for the cache (pydyn recomputes). */
int gb_chemistry(gb_ctx *ctx, const gb_view *temper, const gb_view *phlb, const double *lat,
                 const gb_view *strat_press, const gb_view *strat_oh, const gb_view *strat_cl,
                 const gb_view *strat_od, const gb_view *oh_3d, const gb_view *pl_trop,
                 const gb_view *cl_trop, const gb_view *soil, const double *oh_factor,
                 double oh_scale, double cl_scale, double o1d_scale, double soil_rate,
                 double dt_sec, const int32_t *cols, int ncol, uint32_t tracer_mask,
                 const gb_view *rm, const gb_view *rxm, const gb_view *rym, const gb_view *rzm,
                 const gb_view *krates, double *cache, const int32_t *epoch);
/* The temperature's rate constants of chem.loss_rates (chem.py:137-140) into krates
 * (im, jm, lm, 2): [.., 0] = 2.45e-12 exp(-1775 / T), [.., 1] = (2.36e-12 (T / 298)^1.37)
 * exp(-939 / T), on the listed columns (cols NULL: every column).  A run whose temperature holds
 * for a step makes them once per step for all of its chemistry calls. */
int gb_chem_krates(gb_ctx *ctx, const gb_view *temper, const int32_t *cols, int ncol,
                   const gb_view *krates);
/* sources_region (zoom/physics.py:55-64, emission_data do_add_2d): on the listed columns
 * cols (ncol, 2) int32 device, rm(level, tracer) += x and rzm(level, tracer) -= x, level and
 * tracer 1-based, x = (flux(i, j) area(j)) scale with area (jm) device, or x = flux(i, j) when
 * area is NULL.  rm, rzm (im, jm, lm, nt); flux (im, jm). */
int gb_sources(gb_ctx *ctx, const gb_view *rm, const gb_view *rzm, const gb_view *flux,
               const double *area, double scale, int level, int tracer, const int32_t *cols,
               int ncol);

/* ------------------------------------------------------------------ mass fluxes, pressure
 * dynam0 (kernels.py:102-125, zoom/massflow.py:188-203): am = dt pu, bm = dt pv and cm from the
 * column convergence.  pu (im+1, jm, lm), pv (im, jm+1, lm), bt (lm+1) device; am (im+1, jm, lm),
 * bm (im, jm+1, lm), cm (im, jm, lm+1) destination views. */
int gb_fluxes_from_meteo(gb_ctx *ctx, const gb_view *pu, const gb_view *pv, const double *bt,
                         double dt, const gb_view *am, const gb_view *bm, const gb_view *cm);
/* m2phlb1 / m2phlb (zoom/massflow.py:24-56): sp = seqsum_l(m) g / dxyp(j), phlb = at + bt sp.
 * m (im, jm, lm); sp (im, jm); phlb (im, jm, lm+1); dxyp (jm); at, bt (lm+1).  ring: for a
 * child, the ring cells' p rescaled by dxyp(j) xr yr / dxyp_parent(jpar) -- ring_xr, ring_yr,
 * jbeg and dxyp_parent given (ring_xr = 0: region 1, no rescale). */
int gb_m2phlb(gb_ctx *ctx, const gb_view *m, const gb_view *sp, const gb_view *phlb,
              const double *dxyp, const double *at, const double *bt, int ring_xr, int ring_yr,
              int jbeg, const double *dxyp_parent);

/* The device build of the library's exp / log / pow / cos / sin (op 0..4) on n values: the
 * check that it equals the host build (libgbmath.so) bit for bit; op 5 x / y through the
 * shared-reciprocal division the convection's back substitution uses, op 6 x / y by the
 * hardware division (the check that the two agree), op 7 x / y by the integer-corrected
 * division (div_ip), op 8 x + y and op 9 x - y by the integer-pipe sum (add_ip, sub_ip), op 10
 * sqrt(x) by the integer-corrected root (sqrt_ip), op 11 by the hardware's; Calc_Kzz's flag
 * arithmetic on the integer pipe: op 12 1 x + (1 - 1) y and op 13 0 x + (1 - 0) y (blend01), op 14
 * 0 x (mul01), op 15 jqif(x, y) (jqif_ip).  No reference counterpart. */
int gb_math_eval(gb_ctx *ctx, int op, const double *x, const double *y, double *out, int64_t n);

/* ------------------------------------------------------------------ the adjoint
 * The transposes of a region-1 step's tracer operators with unlimited slopes (limits = 0), for
 * the CH4 surface-flux gradient (one tracer: the adjoint views have nt = 1).  Each call reads
 * the air mass and fluxes the forward operator was given -- taped by the host -- and overwrites
 * the tracer adjoints (rm_b .. rzm_b, the interior (im, jm, lm, 1)) with the adjoints before the
 * operator.  pydyn has no adjoint: these are the transposes of kernels.py:129-346 (dynamu,
 * dynamv, dynamw) and :423-457 (convec), zoom/physics.py:55 (sources_region).
 * gb_adjoint_x: m, am as gb_advect_x got them (am (im+1, jm, lm)), the sub-cycle search redone
 *   as the forward did it; clust as gb_advect_x's.
 * gb_adjoint_y: bm (im, jm+1, lm) before the call, nloop the device int32 per level the forward
 *   returned through its nloop_out.
 * gb_adjoint_z: cm (im, jm, lm+1), n_advz a device int32 (gb_advect_z_last after the forward).
 * gb_adjoint_convec: inv the ncol (lmax x lmax) inverses the forward applied (the cache's).
 * gb_adjoint_sources: grad (im, jm) += area(j) scale (rm_b - rzm_b)(level) on the columns. */
int gb_advect_z_last(gb_ctx *ctx, int32_t *n_out);
int gb_adjoint_x(gb_ctx *ctx, const gb_view *m, const gb_view *rm_b, const gb_view *rxm_b,
                 const gb_view *rym_b, const gb_view *rzm_b, const gb_view *am, const int32_t *clust,
                 int max_nloop);
int gb_adjoint_y(gb_ctx *ctx, const gb_view *m, const gb_view *rm_b, const gb_view *rxm_b,
                 const gb_view *rym_b, const gb_view *rzm_b, const gb_view *bm, const int32_t *nloop);
int gb_adjoint_z(gb_ctx *ctx, const gb_view *m, const gb_view *rm_b, const gb_view *rxm_b,
                 const gb_view *rym_b, const gb_view *rzm_b, const gb_view *cm, const int32_t *n_advz);
int gb_adjoint_convec(gb_ctx *ctx, const gb_view *rm_b, const gb_view *rxm_b, const gb_view *rym_b,
                      const gb_view *rzm_b, const double *inv, const int32_t *cols, int ncol, int lmax);
int gb_adjoint_sources(gb_ctx *ctx, const gb_view *rm_b, const gb_view *rzm_b, const gb_view *grad,
                       const double *area, double scale, int level, const int32_t *cols, int ncol);

/* Measured FP64 issue rate of the device, instructions per second over all SMs: kind 0 a multiply
 * and an add (what -fmad=false emits), 1 a fused multiply-add, 2 a correctly rounded division;
 * kind 3 the multiply with the add on the integer pipe (add_ip; the pair counted as two, as in
 * kind 0), kind 4 the integer-corrected division (div_ip), divisions per second.  The compute
 * ceiling of the float64 step; not capturable.  No reference counterpart. */
int gb_fp64_rate(gb_ctx *ctx, int kind, double *rate);

#ifdef __cplusplus
}
#endif
#endif /* GBDYN_H */
