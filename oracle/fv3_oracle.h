/*
 * fv3_oracle.h -- FP64 CPU restatement of the FV3 tracer-transport path.
 *
 * TEST INFRASTRUCTURE ONLY.  This library is the oracle that the CUDA path in
 * fv3atm_gb300/ is compared against.  Only tests/, __graft_entry__.smoke() and
 * bench.py's CPU-baseline leg may load it.  It is never part of the product.
 *
 * Parity status: UNPINNED.  The upstream Fortran (GFDL_atmos_cubed_sphere,
 * model/tp_core.F90, model/fv_tracer2d.F90, model/fv_mapz.F90) is an empty
 * git submodule in the reference tree (.gitmodules:1-4) and no Fortran compiler
 * exists here, so these routines are restated from the published methods:
 *   - Lin & Rood (1996, MWR 124): flux-form 2-D transport with inner/outer
 *     advective operators;
 *   - Colella & Woodward (1984, JCP 54): PPM, the sub-grid parabola, its
 *     upwind flux integral and the monotonicity constraint (their eq. 1.10);
 *   - Lin (2004, MWR 132): the "fast" monotonicity constraint of the edge
 *     deviations (hord=8) and Lagrangian-to-Eulerian remapping;
 *   - Putman & Lin (2007, JCP 227): one-sided, dxa-weighted edge values at
 *     cube-face edges and the rotated corner fill of the cubed sphere;
 *   - the GFDL_atmos_cubed_sphere tp_core algorithm for the details those
 *     papers leave open: the hord 1 / 5 two-dx filter, the one-sided
 *     interface constants next to a cube edge (s11, s14, s15 for hord 8;
 *     c1, c2, c3 below it), and the deln_flux del-2(nord+1) tracer damping.
 * Call signatures and argument shapes follow the documented FV3 interfaces
 * (fv_tp_2d, tracer_2d, map_scalar, map1_ppm), with Fortran lower bounds given
 * explicitly.  All 2-D arrays are column-major with i fastest.
 */
#ifndef FV3_ORACLE_H
#define FV3_ORACLE_H

#ifdef __cplusplus
extern "C" {
#endif

/* Index bounds of one rank's (or one tile's) domain, as FV3's fv_grid_bounds_type. */
typedef struct {
  int is, ie, js, je;      /* compute domain */
  int isd, ied, jsd, jed;  /* data domain (compute domain + ng halo) */
  int ng;                  /* halo width, 3 */
} orc_bounds;

/* Grid metrics, as the fields of FV3's fv_grid_type that the path reads. */
typedef struct {
  const double* dx;      /* (isd:ied,   jsd:jed+1) length of the south edge   */
  const double* dy;      /* (isd:ied+1, jsd:jed)   length of the west edge    */
  const double* dxa;     /* (isd:ied,   jsd:jed)   cell width along i         */
  const double* dya;     /* (isd:ied,   jsd:jed)   cell width along j         */
  const double* area;    /* (isd:ied,   jsd:jed)                              */
  const double* rarea;   /* (isd:ied,   jsd:jed)   1/area                     */
  const double* sin_sg;  /* (isd:ied,   jsd:jed, 9) slots 1..4 = W,S,E,N edge */
  int sw_corner, se_corner, nw_corner, ne_corner;  /* tile corner is a cube corner */
  int nested;            /* 1: no cube-edge treatment, no corner fill */
  const double* del6_u;  /* (isd:ied,   jsd:jed+1) damping metric of y faces: sina_v dx / dyc */
  const double* del6_v;  /* (isd:ied+1, jsd:jed)   damping metric of x faces: sina_u dy / dxc */
  double da_min;         /* smallest cell area of the cube */
} orc_grid;

/* Cube topology: for tile t and edge e (0=W,1=E,2=S,3=N):
 * topo[(t*4+e)*3 + 0] = neighbour tile, +1 = neighbour edge, +2 = 1 if the
 * along-edge index runs the opposite way on the neighbour. */

/* copy_corners: fill the ng x ng halo blocks at cube corners for a sweep in
 * direction dir (1 = x, 2 = y). */
void orc_copy_corners(double* q, int npx, int npy, int dir, const orc_grid* g, const orc_bounds* bd);

/* fv_tp_2d: fluxes fx (is:ie+1, js:je), fy (is:ie, js:je+1) of one level of
 * one tracer.  q's cube-corner halo blocks are overwritten (copy_corners).
 * hord 1 (with lim_fac), 5 or 8.  mfx/mfy may be NULL (then xfx/yfx weight the
 * fluxes).  damp_c > 1e-4 adds del-2(nord+1) damping fluxes (nord 0..2),
 * weighted by mass (isd:ied, jsd:jed) when mfx is given (mass NULL: none). */
void orc_fv_tp_2d(double* q, const double* crx, const double* cry, int npx, int npy, int hord,
                  double* fx, double* fy, const double* xfx, const double* yfx,
                  const orc_grid* g, const orc_bounds* bd, const double* ra_x, const double* ra_y,
                  double lim_fac, const double* mfx, const double* mfy, const double* mass, int nord,
                  double damp_c);

/* Halo refresh callback used by tracer_2d between substeps (single domain). */
typedef void (*orc_halo_fn)(double* q, int nq, int npz, void* ctx);

/* tracer_2d on one domain (caller refreshes halos through halo_fn, may be NULL
 * when halos are already valid and nsplt == 1).  q (isd:ied,jsd:jed,npz,nq),
 * dp1 (isd:ied,jsd:jed,npz), mfx (is:ie+1,js:je,npz), mfy (is:ie,js:je+1,npz),
 * cx (is:ie+1,jsd:jed,npz), cy (isd:ied,js:je+1,npz).  cx, cy, mfx, mfy are
 * scaled in place by 1/nsplt and dp1 is advanced, as upstream.  Returns nsplt. */
int orc_tracer_2d(double* q, double* dp1, double* mfx, double* mfy, double* cx, double* cy,
                  const orc_grid* g, const orc_bounds* bd, int npx, int npy, int npz, int nq,
                  int hord, int q_split, double dt, int nord_tr, double trdm, double lim_fac,
                  orc_halo_fn halo_fn, void* halo_ctx);

/* Boundary states of a nested grid for one tracer (neststruct%q_BC(iq)) at
 * the parent times t0 and t1, each with npz levels, i fastest:
 *   west (isd:0, jsd:jed)   east (npx:ied, jsd:jed)
 *   south (isd:ied, jsd:0)  north (isd:ied, npy:jed)
 * Only the outer sides of the domain are read. */
typedef struct {
  const double *west_t0, *west_t1, *east_t0, *east_t1;
  const double *south_t0, *south_t1, *north_t0, *north_t1;
} orc_nest_bc;

/* nested_grid_BC_apply_intT for one 3-D field (var (isd:ied,jsd:jed,npz)):
 * the outer-side halo cells become (t0*(split-step) + step*t1)/split. */
void orc_nest_bc_apply(double* var, const orc_bounds* bd, int npx, int npy, int npz, const orc_nest_bc* bc,
                       double step, double split);

/* tracer_2d_nested: tracer_2d whose substeps, on a nested grid (g->nested),
 * apply the boundary states q_bc[0..nq) after halo_fn, with step =
 * *nest_timestep and split = nsplt*k_split; *nest_timestep advances by one
 * per substep of a nested grid.  Returns nsplt. */
int orc_tracer_2d_nested(double* q, double* dp1, double* mfx, double* mfy, double* cx, double* cy,
                         const orc_grid* g, const orc_bounds* bd, int npx, int npy, int npz, int nq,
                         int hord, int q_split, double dt, int nord_tr, double trdm, int k_split,
                         const orc_nest_bc* q_bc, int* nest_timestep, double lim_fac,
                         orc_halo_fn halo_fn, void* halo_ctx);

/* tracer_2d_1L: the levels one at a time, each with its own substep count
 * (q_split > 0, or 1 + the level's Courant maximum) and its fluxes scaled by
 * its own 1/nsplt; halo_fn runs before every substep of every level.
 * nsplt_levels (npz, may be NULL) receives the counts; returns their maximum. */
int orc_tracer_2d_1L(double* q, double* dp1, double* mfx, double* mfy, double* cx, double* cy,
                     const orc_grid* g, const orc_bounds* bd, int npx, int npy, int npz, int nq,
                     int hord, int q_split, double dt, int nord_tr, double trdm, double lim_fac,
                     orc_halo_fn halo_fn, void* halo_ctx, int* nsplt_levels);

/* Fill the edge halo strips of six tiles (all levels/tracers stacked in nplanes
 * planes of (isd:ied, jsd:jed) per tile; tile stride = nplanes planes). */
void orc_cube_halo_fill(double* q, int n, int ng, int nplanes, const int* topo);

/* tracer_2d on the full six-tile cube (arrays have a leading tile dimension of
 * 6 as the OUTERMOST index).  The halo is refreshed from the neighbouring
 * tiles before every substep; every shared tile-edge flux is taken from the
 * lower-numbered tile so global tracer mass is conserved exactly. */
int orc_tracer_2d_cube(double* q, double* dp1, double* mfx, double* mfy, double* cx, double* cy,
                       const orc_grid* g6, int n, int npz, int nq, int hord, int q_split,
                       const int* topo, int sync_edges, int nord_tr, double trdm, double lim_fac);

/* cs_profile / ppm_profile of one column: a4 = (mean, left, right, a6) per
 * layer, a4[4*k + 0..3].  delp > 0 for km layers. */
void orc_column_profile(const double* q, const double* delp, int km, int iv, int kord,
                        double qs, double q_min, double* a4);

/* Remap one column: q1 on pe1 (km+1) -> q2 on pe2 (kn+1). */
void orc_remap_column(int km, const double* pe1, const double* q1, double qs, int kn,
                      const double* pe2, double* q2, int iv, int kord, double q_min);

/* map_scalar / map1_ppm (row j of a 3-D field). */
void orc_map_scalar(int km, const double* pe1, const double* q1, const double* qs, int kn,
                    const double* pe2, double* q2, int i1, int i2, int j, int ibeg, int iend,
                    int jbeg, int jend, int iv, int kord, double q_min);
void orc_map1_ppm(int km, const double* pe1, const double* q1, const double* qs, int kn,
                  const double* pe2, double* q2, int i1, int i2, int j, int ibeg, int iend,
                  int jbeg, int jend, int iv, int kord);

/* Remap every column of nplanes-stacked fields: q1 (ncol, km) column-major
 * i.e. q1[c + k*ncol], pe1 [c + k*ncol] (km+1), pe2 (kn+1). */
void orc_remap_columns(int ncol, int km, const double* pe1, const double* q1, const double* qs,
                       int kn, const double* pe2, double* q2, int iv, int kord, double q_min);

/* Tangent-linear of orc_remap_columns (limiter branches frozen at q1). */
void orc_remap_columns_tl(int ncol, int km, const double* pe1, const double* q1, const double* dq1, const double* qs,
                          int kn, const double* pe2, double* q2, double* dq2, int iv, int kord, double q_min);

/* fillz negative filler, column-mass conserving: q (im, km, nq) inout, dp (im, km). */
void orc_fillz(int im, int km, int nq, double* q, const double* dp);

/* pe, peln, pk (im, km+1) and pkz (im, km) of columns with thickness delp (im, km). */
void orc_pressure_vars(int im, int km, double ptop, double akap, const double* delp, double* pe, double* peln,
                       double* pk, double* pkz);

/* Neumaier-compensated sum of a[i]*b[i]*c[i % nc] over n items. */
double orc_mass_sum(const double* q, const double* dp, const double* area, long n, long narea);

/* Tangent-linear / adjoint of fv_tp_2d with every limiter branch frozen at the
 * trajectory q (hord 5 has none).  dq, dfx/dfy follow the fv_tp_2d shapes. */
void orc_fv_tp_2d_tl(const double* q, const double* dq, const double* crx, const double* cry,
                     int npx, int npy, int hord, double* dfx, double* dfy, const double* xfx,
                     const double* yfx, const orc_grid* g, const orc_bounds* bd,
                     const double* ra_x, const double* ra_y, double lim_fac, const double* mfx,
                     const double* mfy, const double* mass, int nord, double damp_c);

/* Operation counts (counts[0..3] = add/sub, mul, div, min/max/sign) of one
 * fv_tp_2d call (q not modified) and of one column remap, on the tracer-valued
 * quantities: the figure behind the flop ceiling of the measurement. */
void orc_count_fv_tp_2d(const double* q, const double* crx, const double* cry, int npx, int npy, int hord,
                        const double* xfx, const double* yfx, const orc_grid* g, const orc_bounds* bd,
                        const double* ra_x, const double* ra_y, const double* mfx, const double* mfy,
                        unsigned long long* counts);
void orc_count_remap_column(int km, const double* pe1, const double* q1, int kn, const double* pe2, int iv,
                            int kord, unsigned long long* counts);

#ifdef __cplusplus
}
#endif
#endif
