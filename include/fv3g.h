/*
 * fv3g.h -- C ABI of the GB300 (sm_103a) FV3 tracer-transport path.
 *
 * Drop-in for the FV3 dynamical core's tracer transport: horizontal PPM
 * advection (tracer_2d / fv_tp_2d with xppm/yppm and copy_corners) and the
 * Lagrangian-to-Eulerian vertical remap (map_scalar / map1_ppm / cs_profile).
 * The upstream Fortran lives in the GFDL_atmos_cubed_sphere submodule
 * (model/fv_tracer2d.F90, model/tp_core.F90, model/fv_mapz.F90), which is an
 * empty directory in the fv3atm tree (.gitmodules:1-4; linked as CMake target
 * fv3, CMakeLists.txt:43,149).  Its caller in fv3atm is
 * atmosphere_dynamics (atmos_model.F90:879); tracers are stored
 * q(isd:ied, jsd:jed, npz, nq) with i fastest (atmos_model.F90:1423).
 *
 * Conventions
 *  - Everything is plain C: pointers, sizes and doubles/ints, callable from
 *    Fortran through ISO_C_BINDING bind(C) interfaces.
 *  - Arrays passed to the exact-shape entries are HOST arrays in Fortran
 *    (column-major, i fastest) order with the bounds documented per argument;
 *    the library copies them to the GPU and back.
 *  - Every entry returns 0 on success or a negative FV3G_E* code; the message
 *    of the last error on the calling thread is available from
 *    fv3g_last_error().  No entry aborts the process.
 *  - The library never frees caller memory.  Device state is owned by the
 *    opaque fv3g_state handle.
 */
#ifndef FV3G_H
#define FV3G_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ----------------------------------------------------------- error codes -- */
#define FV3G_OK 0
#define FV3G_E_ARG -1        /* bad argument (shape, option, null pointer) */
#define FV3G_E_CUDA -2       /* a CUDA runtime call failed */
#define FV3G_E_COURANT -3    /* Courant number above the supported limit */
#define FV3G_E_NONFINITE -4  /* non-finite value in an input field */
#define FV3G_E_DELP -5       /* a layer thickness became non-positive */
#define FV3G_E_UNSUPPORTED -6 /* option outside the implemented set */
#define FV3G_E_NOMEM -7      /* device allocation failed */
#define FV3G_E_CHECKSUM -8   /* a restart variable's data disagree with its checksum attribute */

/* ------------------------------------------------------------ precision -- */
#define FV3G_FP64 0   /* FP64 throughout */
#define FV3G_MIXED 1  /* FP32 stencils; FP64 pe/peln, remap cumulative mass, mass sums */

/* Bounds of one rank's domain, as FV3's fv_grid_bounds_type. */
typedef struct {
  int is, ie, js, je;     /* compute domain */
  int isd, ied, jsd, jed; /* data domain = compute domain + ng */
  int ng;                 /* halo width; must be 3 */
} fv3g_bounds;

/* Grid metrics (host pointers, FP64), the fields of fv_grid_type on the path. */
typedef struct {
  const double* dx;     /* (isd:ied,   jsd:jed+1) */
  const double* dy;     /* (isd:ied+1, jsd:jed)   */
  const double* dxa;    /* (isd:ied,   jsd:jed)   */
  const double* dya;    /* (isd:ied,   jsd:jed)   */
  const double* area;   /* (isd:ied,   jsd:jed)   */
  const double* rarea;  /* (isd:ied,   jsd:jed)   */
  const double* sin_sg; /* (isd:ied,   jsd:jed, 9) */
  int sw_corner, se_corner, nw_corner, ne_corner; /* tile corner is a cube corner */
  int nested;           /* 1: no cube-edge treatment and no corner fill */
  const double* del6_u; /* (isd:ied,   jsd:jed+1) tracer-damping metric of y faces (sina_v dx / dyc);
                           may be NULL when no damping is asked for */
  const double* del6_v; /* (isd:ied+1, jsd:jed)   of x faces (sina_u dy / dxc) */
  double da_min;        /* smallest cell area of the cube (gridstruct%da_min) */
} fv3g_grid;

/* Halo refresh called by fv3g_tracer_2d before every substep with the HOST
 * tracer array q(isd:ied,jsd:jed,npz,nq); the Fortran side wraps FMS
 * mpp_update_domains here.  May be NULL when halos are valid and nsplt == 1. */
typedef void (*fv3g_halo_fn)(double* q, int nq, int npz, void* ctx);

/* ------------------------------------------------ library / diagnostics -- */
int fv3g_version(void);                      /* 100*major + minor */
int fv3g_last_error(char* buf, int len);     /* copies the calling thread's last message */
int fv3g_device_info(char* buf, int len);    /* GPU name and SM count */

/* ======================================================================== */
/* Exact-shape drop-in entries (host arrays, one domain).                   */
/* ======================================================================== */

/* fv_tp_2d (tp_core.F90): fluxes of one level of one tracer.
 *   q   (isd:ied, jsd:jed)      inout: cube-corner halo blocks are rewritten
 *   crx (is:ie+1, jsd:jed)   cry (isd:ied, js:je+1)
 *   fx  (is:ie+1, js:je)     fy  (is:ie, js:je+1)        out
 *   xfx (is:ie+1, jsd:jed)   yfx (isd:ied, js:je+1)
 *   ra_x (is:ie, jsd:jed)    ra_y (isd:ied, js:je)
 *   mfx (is:ie+1, js:je)     mfy (is:ie, js:je+1)   may be NULL (then xfx/yfx weight the fluxes)
 *   mass (isd:ied, jsd:jed)  may be NULL
 *   hord: 8 (PPM, Lin 2004 monotone constraint), 5 (fourth-order PPM with the
 *   2-dx filter) or 1 (as 5 with the filter test |lim_fac b0| < |bl - br|);
 *   lim_fac is read by hord 1 only, as upstream.
 *   damp_c > 1e-4 adds del-2(nord+1) damping fluxes (deln_flux; nord 0..2,
 *   damp = (damp_c da_min)^(nord+1)): with mfx given only when mass is given,
 *   mass-weighted; without mfx, unweighted.  Damping needs grid->del6_u/v.
 * Replaces: fv_tp_2d(q, crx, cry, npx, npy, hord, fx, fy, xfx, yfx, gridstruct,
 *           bd, ra_x, ra_y, lim_fac, mfx, mfy, mass, nord, damp_c). */
int fv3g_fv_tp_2d(double* q, const double* crx, const double* cry, int npx, int npy, int hord,
                  double* fx, double* fy, const double* xfx, const double* yfx,
                  const fv3g_grid* grid, const fv3g_bounds* bd, const double* ra_x,
                  const double* ra_y, double lim_fac, const double* mfx, const double* mfy,
                  const double* mass, int nord, double damp_c);

/* tracer_2d (fv_tracer2d.F90) on one domain, FP64.
 *   q   (isd:ied, jsd:jed, npz, nq) inout     dp1 (isd:ied, jsd:jed, npz) inout
 *   mfx (is:ie+1, js:je, npz)  mfy (is:ie, js:je+1, npz)                 inout (scaled by 1/nsplt)
 *   cx  (is:ie+1, jsd:jed, npz) cy (isd:ied, js:je+1, npz)               inout (scaled by 1/nsplt)
 *   q_split > 0 fixes the substep count, 0 derives it from the max Courant
 *   number.  hord and lim_fac as fv3g_fv_tp_2d.  trdm > 1e-4 damps the first
 *   substep with del-2(nord_tr+1) fluxes weighted by dp1 (nord_tr 0..2).
 * On return dp1 holds the layer thickness at the start of the last substep,
 * as upstream.  nsplt_out (may be NULL) receives the substep count.
 * Replaces: tracer_2d(q, dp1, mfx, mfy, cx, cy, gridstruct, bd, domain, npx,
 *           npy, npz, nq, hord, q_split, dt, id_divg, q_pack, dp1_pack,
 *           nord_tr, trdm, lim_fac). */
int fv3g_tracer_2d(double* q, double* dp1, double* mfx, double* mfy, double* cx, double* cy,
                   const fv3g_grid* grid, const fv3g_bounds* bd, int npx, int npy, int npz, int nq,
                   int hord, int q_split, double dt, int nord_tr, double trdm, double lim_fac,
                   fv3g_halo_fn halo_fn, void* halo_ctx, int* nsplt_out);

/* tracer_2d_1L (fv_tracer2d.F90; used with fv_core_nml z_tracer): as
 * fv3g_tracer_2d, but the levels are advanced one at a time, each with its
 * own substep count (q_split > 0, or 1 + that level's Courant maximum) and its
 * cx, cy, mfx, mfy scaled by its own 1/nsplt; halo_fn runs before every
 * substep of every level (only that level's planes change in between).
 * nsplt_out receives the largest count.
 * Replaces: tracer_2d_1L(q, dp1, mfx, mfy, cx, cy, gridstruct, bd, domain,
 *           npx, npy, npz, nq, hord, q_split, dt, id_divg, q_pack, dp1_pack,
 *           nord_tr, trdm, lim_fac). */
int fv3g_tracer_2d_1L(double* q, double* dp1, double* mfx, double* mfy, double* cx, double* cy,
                      const fv3g_grid* grid, const fv3g_bounds* bd, int npx, int npy, int npz, int nq,
                      int hord, int q_split, double dt, int nord_tr, double trdm, double lim_fac,
                      fv3g_halo_fn halo_fn, void* halo_ctx, int* nsplt_out);

/* Boundary states of a nested grid for one tracer, neststruct%q_BC(iq), at
 * the parent times t0 and t1 (HOST pointers, i fastest, npz levels each), as
 * allocate_fv_nest_BC_type lays them out for an unstaggered field
 * (moving_nest/fv_moving_nest.F90:2005-2008):
 *   west  (isd:0,   jsd:jed, npz)   read when is == 1
 *   east  (npx:ied, jsd:jed, npz)   read when ie == npx-1
 *   south (isd:ied, jsd:0,   npz)   read when js == 1
 *   north (isd:ied, npy:jed, npz)   read when je == npy-1
 * South and north are read over i = is..ie on an outer side of the domain
 * and to isd/ied toward a neighbour rank; the corner blocks come from west and
 * east.  The strips of a side that is not read may be NULL. */
typedef struct {
  const double *west_t0, *west_t1, *east_t0, *east_t1;
  const double *south_t0, *south_t1, *north_t0, *north_t1;
} fv3g_nest_bc;

/* tracer_2d_nested (fv_tracer2d.F90; the variant fv_dynamics calls on a
 * nested grid or on a grid with nests): fv3g_tracer_2d, and on a nested grid
 * (grid->nested = 1) the halo cells on the domain's outer sides are set before
 * every substep, after halo_fn, from q_bc[0..nq) interpolated in time as
 *   q = (t0*(split - step) + step*t1) * (1/split),
 *   split = nsplt*k_split, step = *nest_timestep,
 * the count of tracer substeps taken since the parent's t0
 * (neststruct%tracer_nest_timestep, moving_nest/fv_moving_nest.F90:1781);
 * it advances by one per substep and is written back on success.  On a grid
 * that is not nested q_bc may be NULL and the count is left as it is.
 * Replaces (argument list as documented upstream): tracer_2d_nested(q, dp1,
 *           mfx, mfy, cx, cy, gridstruct, bd, domain, npx, npy, npz, nq,
 *           hord, q_split, dt, id_divg, q_pack, dp1_pack, nord_tr, trdm,
 *           k_split, neststruct, parent_grid, n_map, lim_fac). */
int fv3g_tracer_2d_nested(double* q, double* dp1, double* mfx, double* mfy, double* cx, double* cy,
                          const fv3g_grid* grid, const fv3g_bounds* bd, int npx, int npy, int npz, int nq,
                          int hord, int q_split, double dt, int nord_tr, double trdm, int k_split,
                          const fv3g_nest_bc* q_bc, int* nest_timestep, double lim_fac,
                          fv3g_halo_fn halo_fn, void* halo_ctx, int* nsplt_out);

/* map_scalar (fv_mapz.F90): remap row j of a 3-D field, FP64.
 *   pe1 (i1:i2, km+1)  pe2 (i1:i2, kn+1)  qs (i1:i2)
 *   q1 (ibeg:iend, jbeg:jend, km) in    q2 (ibeg:iend, jbeg:jend, kn) inout
 *   iv: -2 (bottom value qs, which must then be given), -1, 0 (positive), 1 (floor q_min)
 *   kord: 4 (C1 spline, CW84 limiter) or 9 (monotone)
 *   pe2(1) must equal pe1(1) and pe2(kn+1) must equal pe1(km+1).
 * Thread-safe: may be called concurrently from OpenMP threads (per-thread
 * stream and scratch).
 * Replaces: map_scalar(km, pe1, q1, qs, kn, pe2, q2, i1, i2, j, ibeg, iend,
 *           jbeg, jend, iv, kord, q_min). */
int fv3g_map_scalar(int km, const double* pe1, const double* q1, const double* qs, int kn,
                    const double* pe2, double* q2, int i1, int i2, int j, int ibeg, int iend,
                    int jbeg, int jend, int iv, int kord, double q_min);

/* map1_q2 (fv_mapz.F90): the map1_ppm reconstruction of row j of q1 onto the
 * target interfaces pe2, with the target thicknesses dp2 (i1:i2, kn) given:
 * a target layer spanning several source layers takes its overlap mass
 * divided by dp2; q2 is the 2-D row (i1:i2, kn).  q_min: the floor of iv 1.
 * Replaces: map1_q2(km, pe1, q1, kn, pe2, q2, dp2, i1, i2, iv, kord, j, ibeg,
 *           iend, jbeg, jend, q_min). */
int fv3g_map1_q2(int km, const double* pe1, const double* q1, int kn, const double* pe2, double* q2,
                 const double* dp2, int i1, int i2, int iv, int kord, int j, int ibeg, int iend, int jbeg, int jend,
                 double q_min);

/* map1_ppm (fv_mapz.F90): as map_scalar without the floor argument.
 * Replaces: map1_ppm(km, pe1, q1, qs, kn, pe2, q2, i1, i2, j, ibeg, iend,
 *           jbeg, jend, iv, kord). */
int fv3g_map1_ppm(int km, const double* pe1, const double* q1, const double* qs, int kn,
                  const double* pe2, double* q2, int i1, int i2, int j, int ibeg, int iend,
                  int jbeg, int jend, int iv, int kord);

/* Whole-domain remap of nq fields in one call (the loop over j rows and
 * tracers of Lagrangian_to_Eulerian / mapn_tracer, fv_mapz.F90):
 *   pe1 (i1:i2, j1:j2, km+1)  pe2 (i1:i2, j1:j2, kn+1)  qs (i1:i2, j1:j2) or NULL
 *   q1 (ibeg:iend, jbeg:jend, km, nq) in    q2 (ibeg:iend, jbeg:jend, kn, nq) inout */
int fv3g_map_scalar_3d(int km, const double* pe1, const double* q1, const double* qs, int kn,
                       const double* pe2, double* q2, int i1, int i2, int j1, int j2, int ibeg,
                       int iend, int jbeg, int jend, int nq, int iv, int kord, double q_min);

/* ------------------------------------------------------------------------ */
/* Tangent-linear and adjoint models (tp_core / fv_mapz TL-AD pairs): the    */
/* derivative with respect to the tracer only -- Courant numbers, mass       */
/* fluxes and pressures frozen -- with every limiter branch frozen at the    */
/* trajectory q.  Adjoints follow the generated-code convention: input       */
/* adjoints are incremented, output adjoints are consumed (set to zero).     */
/* ------------------------------------------------------------------------ */

/* fv_tp_2d tangent-linear: (q, q_tl) -> (fx, fx_tl, fy, fy_tl); q and q_tl
 * are read only (the copy_corners side effect on q is not reproduced);
 * fx / fy may be NULL.  Other arguments as fv3g_fv_tp_2d. */
int fv3g_fv_tp_2d_tl(const double* q, const double* q_tl, const double* crx, const double* cry, int npx,
                     int npy, int hord, double* fx, double* fx_tl, double* fy, double* fy_tl,
                     const double* xfx, const double* yfx, const fv3g_grid* grid, const fv3g_bounds* bd,
                     const double* ra_x, const double* ra_y, double lim_fac, const double* mfx,
                     const double* mfy, const double* mass, int nord, double damp_c);

/* fv_tp_2d adjoint at trajectory q: q_ad (isd:ied, jsd:jed) += J^T (fx_ad, fy_ad);
 * fx_ad (is:ie+1, js:je) and fy_ad (is:ie, js:je+1) are set to zero.
 * Damping (damp_c > 1e-4 where it applies) is differentiated for nord 0
 * (del-2); higher orders return FV3G_E_UNSUPPORTED. */
int fv3g_fv_tp_2d_ad(const double* q, double* q_ad, const double* crx, const double* cry, int npx, int npy,
                     int hord, double* fx_ad, double* fy_ad, const double* xfx, const double* yfx,
                     const fv3g_grid* grid, const fv3g_bounds* bd, const double* ra_x, const double* ra_y,
                     double lim_fac, const double* mfx, const double* mfy, const double* mass, int nord,
                     double damp_c);

/* map1_ppm tangent-linear on row j: (q1, q1_tl) -> (q2, q2_tl); q2 may be NULL. */
int fv3g_map1_ppm_tl(int km, const double* pe1, const double* q1, const double* q1_tl, const double* qs,
                     int kn, const double* pe2, double* q2, double* q2_tl, int i1, int i2, int j, int ibeg,
                     int iend, int jbeg, int jend, int iv, int kord);

/* map1_ppm adjoint on row j at trajectory q1: q1_ad += J^T q2_ad; q2_ad = 0. */
int fv3g_map1_ppm_ad(int km, const double* pe1, const double* q1, double* q1_ad, const double* qs, int kn,
                     const double* pe2, double* q2_ad, int i1, int i2, int j, int ibeg, int iend, int jbeg,
                     int jend, int iv, int kord);

/* fillz (fv_fill.F90): negative tracer values filled column by column,
 * conserving each column's mass.  q (im, km, nq) inout, dp (im, km) in.
 * Replaces: fillz(im, km, nq, q, dp). */
int fv3g_fillz(int im, int km, int nq, double* q, const double* dp);

/* Pressure variables after the remap (the pe/peln/pk/pkz recompute of
 * Lagrangian_to_Eulerian): pe = ptop + running sum of delp, peln = ln pe,
 * pk = pe^akap, pkz = (pk(k+1) - pk(k)) / (akap (peln(k+1) - peln(k))).
 * delp (im, km) in; pe, peln, pk (im, km+1) and pkz (im, km) out. */
int fv3g_pressure_vars(int im, int km, double ptop, double akap, const double* delp, double* pe, double* peln,
                       double* pk, double* pkz);

/* Column remap on caller-owned DEVICE arrays that allocates no device memory.
 * No counterpart in the reference: it serves callers that cannot let a
 * library call cudaMalloc/cudaFree -- a model that owns all of its device
 * memory (e.g. Fortran ported with OpenACC, passing device pointers through
 * host_data use_device) or code that must not take the implicit device
 * synchronisation of an allocation inside its time loop.
 *   pe1 [km+1][ncol], pe2 [kn+1][ncol], q1 [nfield][km][ncol],
 *   q2 [nfield][kn][ncol], qs [ncol] or NULL; FP64, device pointers.
 *   iv, kord, q_min as fv3g_map_scalar; stream: CUDA stream, NULL = default.
 * Limits: ncol <= 1024 and km, kn <= 128 per call; larger requests return
 * FV3G_E_ARG.  The scratch is one fixed device array (6.5 MB, kept by every
 * GPU that loads the library until exit) shared by all calls, so calls that
 * overlap on the GPU (on different streams or host threads) race; serialise
 * them.  The first call on each device looks up the array's device address
 * (cudaGetSymbolAddress); make that first call before any stream capture.
 * The looked-up addresses are kept for the life of the process: resetting a
 * device (cudaDeviceReset) after the first call is not supported.
 * iv == -2 needs qs (FV3G_E_ARG otherwise). */
int fv3g_remap_columns_noalloc(int ncol, int km, const double* pe1, const double* q1, const double* qs,
                               int kn, const double* pe2, double* q2, int nfield, int iv, int kord,
                               double q_min, void* stream);

/* ======================================================================== */
/* Batched, device-resident entries (all six tiles, all tracers).           */
/* ======================================================================== */

typedef struct fv3g_state fv3g_state;

typedef struct {
  int n;          /* cells per tile edge (C_n) */
  int ntiles;     /* 6: the cube, halos from the neighbouring tiles; 1: one cube face whose halo ring
                     (strips and corner blocks of Q) is uploaded by the caller and held over the step;
                     with independent_tiles, any count of such single faces (members of one size) */
  int npz;        /* Lagrangian levels */
  int nq;         /* tracers */
  int precision;  /* FV3G_FP64 or FV3G_MIXED */
  int hord;       /* 1, 5 or 8 (see fv3g_fv_tp_2d) */
  int kord;       /* 4 or 9 */
  int iv;         /* remap iv (see fv3g_map_scalar): -1, 0 or 1; -2 needs a per-column qs, which a state does not hold */
  double q_min;   /* remap floor for iv == 1 */
  int warps_per_cta; /* advection CTA width in warps (0 = default) */
  int nord_tr;    /* tracer damping order 0..2 (del-2(nord_tr+1)) */
  double trdm;    /* damping coefficient; > 1e-4 damps the first substep (needs the grid's del6_u/v) */
  double lim_fac; /* hord 1 filter factor; 0 means 1 */
  int fill;       /* 1: fillz the remapped tracers in every remap (fv_core_nml fill) */
  int edge_sync;  /* six tiles: 1 makes each shared tile-edge face carry one flux, the upwind tile's (the
                     downwind tile's edge cell is corrected); 0 (upstream behaviour) keeps each tile's own
                     value.  With halos that hold the neighbours' cells, metrics and winds the two values
                     already agree to round-off; the option removes that round-off from the global mass. */
  int mass_fix;   /* 1: after every remap of all tiles, restore each tracer's global mass sum(q delp area) to its
                     value at the step's start (the transport conserves it; FP32 storage rounds it by ~1e-10 per
                     step): FP64 states scale q by (1 + eps); FP32 states move a dithered few values (in a fixed
                     1/16 of the rows) by one unit in the last place, unbiased, then a few small values to take
                     the residual to ~1e-14 (the stored FP32 mass is summed exactly).  Switchable per step with
                     fv3g_state_set_mass_fix. */
  int independent_tiles; /* 1: the ntiles tiles are independent single faces (ensemble members of one size and
                     level count, each with its own grid, fields and prescribed halo ring), advanced together:
                     one launch per phase for all of them; 0: ntiles 6 is the cube, 1 one face */
} fv3g_state_desc;

/* Which field an upload/download addresses. */
enum {
  FV3G_FIELD_Q = 0,    /* (6, nq, npz, nd, nd)    nd = n + 6, halo included */
  FV3G_FIELD_DELP,     /* (6, npz, nd, nd)        Lagrangian thickness at call start */
  FV3G_FIELD_CX,       /* (6, npz, nd, n+1)       Fortran (is:ie+1, jsd:jed) per level */
  FV3G_FIELD_CY,       /* (6, npz, n+1, nd)       (isd:ied, js:je+1) */
  FV3G_FIELD_MFX,      /* (6, npz, n, n+1)        (is:ie+1, js:je) */
  FV3G_FIELD_MFY,      /* (6, npz, n+1, n)        (is:ie, js:je+1) */
  FV3G_FIELD_Q_REMAPPED, /* (6, nq, npz, nd, nd) output of the remap */
  FV3G_FIELD_DELP_OUT,   /* (6, npz, nd, nd)      thickness after the last substep */
  FV3G_NFIELDS
};

/* Grid of one tile (host arrays with the fv3g_grid shapes, tile-local bounds). */
int fv3g_state_create(const fv3g_state_desc* desc, fv3g_state** out);
int fv3g_state_destroy(fv3g_state* st);
int fv3g_state_set_grid(fv3g_state* st, int tile, const fv3g_grid* grid);
int fv3g_state_set_levels(fv3g_state* st, const double* ak, const double* bk); /* npz+1 each */
/* Host <-> device copies (FP64 host data; converted to FP32 in MIXED mode).
 * Every `stream` argument of this header: NULL selects the state's own
 * (non-blocking) stream; any other handle is used as given, including
 * cudaStreamLegacy ((void*)1) for the legacy default stream.  Work on a
 * stream other than the state's (copies, steps, remaps, mass sums, the
 * ensemble step) is ordered after the work already queued on the state's
 * stream and before the work queued there after it; a stream under capture
 * is left to the caller that builds the graph. */
int fv3g_upload(fv3g_state* st, int field, const double* host);
int fv3g_download(fv3g_state* st, int field, double* host);
/* Raw device copies with the state's storage type (float in MIXED). */
int fv3g_upload_device(fv3g_state* st, int field, const void* dptr, void* stream);
int fv3g_download_device(fv3g_state* st, int field, void* dptr, void* stream);

/* One tracer_2d call on device data: nsplt = q_split (1..64), or with
 * q_split = 0 tracer_2d's int(1 + max |Courant|) over every tile's compute
 * cells of CX and CY (one device-to-host read, so the call waits for the
 * stream; FV3G_E_NONFINITE / FV3G_E_COURANT for a non-finite maximum or a
 * count above 64).  fv3g_state_nsplt returns the count used last. */
int fv3g_tracer_2d_batched(fv3g_state* st, int q_split, void* stream);
int fv3g_state_nsplt(fv3g_state* st, int* nsplt);
/* Remap every tracer from the Lagrangian levels of DELP_OUT to ak + bk*ps. */
int fv3g_remap_batched(fv3g_state* st, void* stream);
/* The remap of Lagrangian_to_Eulerian for fields beside the tracers (pt and
 * the winds), from the Lagrangian levels of the last tracer_2d (DELP_OUT) onto
 * ak + bk ps: nfield fields in device arrays of the state's element type in
 * the layout of FV3G_FIELD_Q ((ntiles, nfield, npz) planes of nd x nd); only
 * the kind's columns are read and written.
 *   kind 0: cell-centred fields (pt with iv 1 and q_min its floor, kord_tm);
 *     log_p 1 remaps in ln p, as pt is remapped on peln;
 *   kind 1: u winds on the y faces (i = 1..n, j = 1..n+1), kind 2: v winds on
 *     the x faces (i = 1..n+1, j = 1..n), each face column's pressures the
 *     mean of the two cells beside it (iv -1, kord_mt); six-tile cube only.
 * Replaces: the pt, u and v remaps of Lagrangian_to_Eulerian (fv_mapz.F90:
 *   map_scalar on peln for pt, map1_ppm with pe0 / pe3 for u and v). */
int fv3g_state_remap_fields(fv3g_state* st, const void* fields_in, void* fields_out, int nfield, int kind, int iv,
                            int kord, double q_min, int log_p, void* stream);
/* Tangent-linear and adjoint of one step (tracer_2d with q_split substeps,
 * then the remap; parts = 1: tracer_2d alone (output on the Lagrangian
 * levels), 2: the remap alone (of the home field on DELP), 3: both) of an
 * FP64 six-tile state about its current inputs (the
 * home tracer field Q, DELP, CX, CY, MFX, MFY and the levels), with the
 * winds and thicknesses frozen and every limiter branch frozen at the
 * trajectory (trdm 0, fill 0, edge_sync 0, mass_fix 0; hord 1, 5 or 8).
 * Each call runs the forward substeps and keeps every substep's input as a
 * checkpoint, from which the linearised substeps recompute their trajectory.
 * Arrays are device pointers in the layout of FV3G_FIELD_Q (nt*nq*npz planes
 * of nd x nd, i fastest); only interior cells are read, and halo cells of the
 * outputs are zero.
 *   fv3g_state_step_tl: dq_out = J dq_in (kord 4 or 9: the remap runs as the
 *     remap kernel on value/tangent pairs).
 *   fv3g_state_step_ad: q_ad_in = J^T q_ad_out (hand-written reverse sweeps:
 *     the substeps' PPM stencils, copy_corners and the cube halo transposed,
 *     and the kord-4 column remap; kord 9 returns FV3G_E_UNSUPPORTED).
 * Replace: the tangent-linear / adjoint of tracer_2d (fv_tracer2d.F90) and of
 * the tracer remap of Lagrangian_to_Eulerian (fv_mapz.F90). */
int fv3g_state_step_tl(fv3g_state* st, int q_split, int parts, const double* dq_in, double* dq_out,
                       void* stream);
int fv3g_state_step_ad(fv3g_state* st, int q_split, int parts, const double* q_ad_out, double* q_ad_in,
                       void* stream);
/* tracer_2d + remap; with use_graph the step is captured once as a CUDA graph
 * and replayed on later calls with the same substep count (q_split 0: the
 * count is derived first, as in fv3g_tracer_2d_batched). */
int fv3g_step(fv3g_state* st, int q_split, int use_graph, void* stream);
/* Compensated FP64 global tracer mass sum(q*delp*area) over 6 tiles, per
 * tracer, of the field (FV3G_FIELD_Q with DELP, or Q_REMAPPED with the
 * remapped thickness).  Writes nq doubles to host_out. */
int fv3g_mass_sum(fv3g_state* st, int which, double* host_out, void* stream);
/* Asynchronous copies with the host data type chosen by the caller
 * (host_f32 = 1: float host arrays, as a 32BIT build of the model holds them;
 * 0: double).  An FP64 state needs double host data.  Use pinned host memory
 * for full bandwidth; fv3g_stream_sync waits for them. */
int fv3g_upload_async(fv3g_state* st, int field, const void* host, int host_f32, void* stream);
int fv3g_download_async(fv3g_state* st, int field, void* host, int host_f32, void* stream);
int fv3g_stream_sync(fv3g_state* st, void* stream);
/* One tracer_2d + remap step from host arrays to host arrays with the
 * transfers overlapped with the compute: the tracers move in `groups` groups,
 * and group g is advected and remapped while group g+1 uploads and group g-1
 * downloads; the remap runs tile by tile, each tile's download starting as
 * soon as it is remapped.  On the six-tile cube with q_split given, at least
 * 16 levels, edge_sync 0 and mass_fix 0 the first group's per-level inputs and
 * tracers stream in 8 level blocks, each block advected as soon as it has
 * arrived (groups 0: one group there, else nq / warps_per_cta groups after
 * the per-level inputs).  q_in, q_out: (ntiles, nq, npz, nd, nd); delp, cx, cy, mfx, mfy:
 * the FV3G_FIELD_* shapes; element type float (host_f32 = 1, MIXED states) or
 * double (FP64 states); page-locked host memory for full bandwidth.  With a
 * stream the work is ordered after the stream's prior work and the call
 * returns once it is enqueued (the stream waits for its end); with NULL it
 * returns when q_out holds the result.  q_split 0 derives the substep count
 * from the uploaded Courant numbers (the call then waits for the per-level
 * uploads before it enqueues the rest). */
int fv3g_step_host(fv3g_state* st, int q_split, const void* q_in, const void* delp, const void* cx,
                   const void* cy, const void* mfx, const void* mfy, void* q_out, int host_f32,
                   int groups, void* stream);
/* Choose the advection CTA width (warps per CTA) by timing one substep of
 * the loaded fields at each candidate width -- for FP32 states with hord 8
 * both with one tracer per warp and with two (fv3g_state_set_tracer_pairs)
 * -- and keep the fastest for the state (warps_out may be NULL).
 * Side-effect free on the state's fields.  Call it outside stream capture,
 * after the inputs are uploaded. */
int fv3g_state_autotune(fv3g_state* st, int* warps_out);
/* FP32 states with hord 8: advance the tracers two per warp (on = 1; packed
 * FP32 pair arithmetic, up to 12 warps per CTA) or one per warp (0, the
 * default).  Results agree to FP32 rounding.  FV3G_E_UNSUPPORTED for other
 * states when on = 1. */
int fv3g_state_set_tracer_pairs(fv3g_state* st, int on);
int fv3g_state_tracer_pairs(fv3g_state* st, int* on);
/* The kernel of the state's remap: 0 (the default) runs every state one
 * warp per column; 1 runs FP32 states with kord 9, iv -1..1 and at least 16
 * levels one thread per column (float-float overlap schedule, the
 * elimination of the interface system recomputed per chunk of levels) and
 * every other state one warp per column.  Both give the same schemes; FP32
 * results agree to rounding.  At 6 x C384 L127 x 20 tracers the warp form
 * takes 36.8 ms per remap, the thread form 56.5 ms. */
int fv3g_state_set_remap_form(fv3g_state* st, int form);
int fv3g_state_remap_form(fv3g_state* st, int* form);
/* Switch the mass fixer (fv3g_state_desc.mass_fix) on (1) or off (0) for
 * the following steps. */
int fv3g_state_set_mass_fix(fv3g_state* st, int on);
/* The advection CTA widths in use: interior CTAs and the CTAs whose window
 * holds a cube-face edge (the autotuner may run those narrower). */
int fv3g_state_widths(fv3g_state* st, int* warps, int* warps_ring);
/* fillz on the state's remapped tracers (every interior column and tracer). */
int fv3g_fillz_batched(fv3g_state* st, void* stream);

/* Ensembles: independent states of any sizes advanced together.  One step
 * runs tracer_2d (q_split substeps) and the remap of every member, as one
 * CUDA graph that forks to a stream per member and joins; members must have
 * their levels set and timing off.  The ensemble does not own its members.
 * The graph runs on `stream` (NULL: the ensemble's own first stream);
 * synchronise that stream, or the device, before reading the members. */
typedef struct fv3g_ensemble fv3g_ensemble;
int fv3g_ensemble_create(fv3g_state* const* members, int n, fv3g_ensemble** out);
int fv3g_ensemble_step(fv3g_ensemble* ens, int q_split, void* stream);
int fv3g_ensemble_destroy(fv3g_ensemble* ens);
/* Per-kernel timing of fv3g_step: with timing enabled, CUDA events are
 * recorded around every kernel of the step (also inside the graph);
 * fv3g_kernel_times returns, for the last completed step, the summed ms and
 * the kernel launch count per kind (arrays of FV3G_KERNEL_KINDS entries):
 * [0] prologue (area fluxes), [1] advection substep, [2] tile-edge flux fix,
 * [3] column remap, [4] halo strips of the six tiles. */
#define FV3G_KERNEL_KINDS 5
int fv3g_set_timing(fv3g_state* st, int enable);
int fv3g_kernel_times(fv3g_state* st, double* ms_by_kind, int* launches_by_kind);
/* Sticky device error word of the state (0 = none), the first of: FV3G_E_NONFINITE
 * (a non-finite Courant number or mass flux on a compute face), FV3G_E_COURANT
 * (a Courant number over q_split above 1 in magnitude), FV3G_E_DELP (a layer
 * thickness not positive after a substep's mass fluxes), raised on the device
 * by the steps since the last read; the step runs to its end regardless.
 * Waits for the work queued on the state's own streams (work queued on a
 * caller's stream must be complete first); cleared by reading. */
int fv3g_state_error(fv3g_state* st, int* code);
/* Device pointer and element strides of a field (for zero-copy harnesses). */
int fv3g_field_info(fv3g_state* st, int field, void** dptr, long long* strides4, int* pitch);

/* ------------------------------------------------------- restart files -- */
/* The restart files of the path, fv_tracer.res.tile<t>.nc (the tracers) and
 * fv_core.res.tile<t>.nc (delp), which fv3atm reads at start-up and writes at
 * restart times (atmos_model.F90:105,1149-1166), in the layout of the write
 * component (io/module_write_restart_netcdf.F90:244-317): dimensions xaxis_1,
 * yaxis_1, zaxis_1 and the unlimited Time, every field (Time, zaxis_1,
 * yaxis_1, xaxis_1) with a 'checksum' attribute, FMS mpp_chksum written as
 * '(Z16)' (:444-530): the sum modulo 2^64 of the values' bit patterns taken
 * as 64-bit integers (FP64 data) or as sign-extended 32-bit integers (FP32).
 * Containers: netCDF classic (CDF-1), 64-bit offset (CDF-2) and 64-bit data
 * (CDF-5).  netCDF-4/HDF5 files are refused with FV3G_E_UNSUPPORTED (convert
 * them with nccopy -k cdf5 first).  Host-side calls (open, info, checksum,
 * read) need no GPU. */
typedef struct fv3g_ncfile fv3g_ncfile;
#define FV3G_NC_FLOAT 5
#define FV3G_NC_DOUBLE 6
int fv3g_nc_open(const char* path, fv3g_ncfile** out);
int fv3g_nc_close(fv3g_ncfile* f);
int fv3g_nc_nvars(fv3g_ncfile* f, int* nvars);
/* Variable idx (0-based): its name (NUL-terminated, cut to len), netCDF type
 * (1 byte ... 6 double, 7..11 the CDF-5 types), rank and shape (slowest
 * first, at most 8 entries written; the record dimension counts the file's
 * records) and whether it is a record variable. */
int fv3g_nc_var_info(fv3g_ncfile* f, int idx, char* name, int len, int* nc_type, int* ndims, long long* shape,
                     int* is_record);
/* The variable's 'checksum' attribute; present = 0 when it has none. */
int fv3g_nc_checksum(fv3g_ncfile* f, const char* name, unsigned long long* checksum, int* present);
/* Host read of one record (ignored for a fixed variable) converted to FP64;
 * count must equal the variable's values per record. */
int fv3g_nc_read(fv3g_ncfile* f, const char* name, int record, double* out, long long count);
/* Load record 0 of nvars variables, each (zaxis, yaxis, xaxis) = (npz, n, n),
 * into tile `tile` (0-based) of a state field: FV3G_FIELD_Q with slots[v]
 * the tracer index of variable v, or FV3G_FIELD_DELP (one variable, slots
 * NULL).  The file's bytes go to the GPU as they are; one kernel swaps the
 * byte order, converts to the state's precision, places the values in the
 * halo-padded planes (halos untouched) and sums the checksum.  verify != 0: a
 * checksum attribute that disagrees fails with FV3G_E_CHECKSUM (fv3atm's
 * ignore_rst_cksum = .false.).  checksums (nvars, may be NULL) receive the
 * sums.  Loading Q makes the latest tracer buffer the home buffer first, so
 * tracers not loaded keep their latest values.  Synchronous. */
int fv3g_state_read_restart(fv3g_state* st, int field, int tile, fv3g_ncfile* f, const char* const* names,
                            const int* slots, int nvars, int verify, unsigned long long* checksums);
/* Write the latest values of tile `tile` of a state field (slots as above)
 * to a new file at path in the write component's layout, as nc_type
 * FV3G_NC_FLOAT or FV3G_NC_DOUBLE in container version 1, 2 or 5 (CDF-1,
 * CDF-2, CDF-5); checksums (nvars, may be NULL) receive the sums written into
 * the attributes.  Synchronous. */
int fv3g_state_write_restart(fv3g_state* st, int field, int tile, const char* path, const char* const* names,
                             const int* slots, int nvars, int nc_type, int version, unsigned long long* checksums);

#ifdef __cplusplus
}
#endif
#endif /* FV3G_H */
