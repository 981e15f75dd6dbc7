/*
 * cans_gb300 -- C ABI of the GB300 (sm_103a) pressure-correction path of CaNS.
 *
 * Every entry point mirrors one routine of the reference Fortran code
 * (file:line cited per declaration) with the same argument meaning, so a
 * Fortran host binds it with an iso_c_binding interface block and passes the
 * device addresses of its `!$acc enter data` arrays (host_data use_device).
 *
 * Conventions
 *   - Fields u, v, w, p, pp are caller-owned DEVICE arrays in Fortran order
 *     with one ghost layer: extents (n1+2, n2+2, n3+2), element (i,j,k),
 *     0 <= i <= n1+1, at offset i + (n1+2)*(j + (n2+2)*k).
 *   - 1D grid arrays dzc, dzf, dzci, dzfi are DEVICE arrays indexed 0..n3+1;
 *     the `_g` arrays passed to cans_initsolver are HOST arrays 0..ng3+1.
 *   - Boundary conditions cbc(0:1,3) are 6 chars in Fortran order
 *     cbc[ibound + 2*idir] ('P','D','N'); velocity cbcvel(0:1,3,3) are 18
 *     chars cbcvel[ibound + 2*idir + 6*icomp]; values bc/bcvel likewise.
 *   - is_bound(0:1,3) is 6 ints, is_bound[ibound + 2*idir].
 *   - `stream` is a cudaStream_t (NULL = legacy default stream).  All calls
 *     are asynchronous on it unless documented otherwise; nothing aborts;
 *     every call returns a status code below.
 *   - A plan is not thread-safe; use one plan per host thread.
 */
#ifndef CANS_GB300_H
#define CANS_GB300_H
#include <stddef.h>
#ifdef __cplusplus
extern "C" {
#endif

/* status codes (the reference ignores istat and uses `error stop`) */
#define CANS_OK 0
#define CANS_EINVAL 1      /* bad argument (sizes, BC characters, NULL pointers) */
#define CANS_ENOMEM 2      /* device allocation failed */
#define CANS_ECUDA 3       /* a CUDA call or kernel launch failed */
#define CANS_ENOTSUP 4     /* transform length (a prime factor above 61) or BC combination not supported */
#define CANS_ETIMEOUT 5    /* a bounded device wait expired */
#define CANS_ENONFINITE 6  /* non-finite value detected in a checked result */
#define CANS_EIO 7         /* a checkpoint file could not be opened, read or written */

/* arithmetic of a plan */
#define CANS_FP64 0        /* all transforms/eliminations in FP64 */
#define CANS_FP32 1        /* FP32 transforms, FP64 tridiagonal elimination */

typedef struct cans_plan cans_plan; /* arrplan + lambdaxy + a,b,c + normfft + work space */

const char *cans_strerror(int status);
/* library build identification (e.g. "cans_gb300 sm_103a") */
const char *cans_version(void);

/* ---- set-up ------------------------------------------------------------------------------ */
/* initgrid (src/initgrid.f90:14-99): HOST arrays dzc, dzf, zc, zf (0..n+1); gtype 1..4
 * (two-end, one-end, one-end reversed, middle clustering) */
int cans_initgrid(int gtype, int n, double gr, double lz, int is_periodic, double *dzc, double *dzf,
                  double *zc, double *zf);
/* initsolver (src/initsolver.f90:15-16) + fftini (src/fft.f90:25-209).
 * Builds the eigenvalues, the z tridiagonal coefficients, the boundary RHS
 * values and the transform plans on the device.  Optional HOST outputs (NULL
 * to skip) return what the reference returns:
 *   lambdaxy[ng1*ng2] (Fortran order), a,b,c[ng3], *normfft,
 *   rhsb[6] = the constant face values of rhsb{x,y,z}(:,:,0:1), rhsb[ibound+2*idir].
 * ng[0], ng[1]: any length whose prime factors are at most 61 (the reference takes any
 * length through FFTW/cuFFT); a larger prime factor returns CANS_ENOTSUP. */
int cans_initsolver(const int ng[3], const double dli[3], const double *dzci_g, const double *dzfi_g,
                    const char cbc[6], const double bc[6], const char c_or_f[3], int precision,
                    void *stream, cans_plan **plan,
                    double *lambdaxy, double *a, double *b, double *c, double *normfft, double rhsb[6]);
/* initflow (src/initflow.f90:16-259), one GPU: the initial u, v, w, p (device, haloed, FP64;
 * interiors written, ghosts untouched) for inivel 'cou' 'poi' 'tbl' 'iop' 'zer' 'uni' 'log'
 * 'hcl' 'hcp' 'tgv' 'tgw' 'ant' 'pdc' 'hdc' (CANS_EINVAL otherwise), with the reference's noise
 * amplitudes, seeds (123, 456, 789), bulk-velocity rescaling and, with is_wallturb, the
 * cross-stream vortex pair.  zc, zf, dzc, dzf: HOST arrays 0..n3+1 (cans_initgrid).  The
 * noise is splitmix64 of (seed, global cell index): the reference's gfortran random_number
 * stream cannot be reproduced.  Synchronises `stream`. */
int cans_initflow(const char inivel[3], const double bcvel[18], const int n[3], const double l[3],
                  const double dl[3], const double *zc, const double *zf, const double *dzc,
                  const double *dzf, double visc, const int is_forced[3], const double velf[3],
                  const double bforce[3], int is_wallturb, double *u, double *v, double *w, double *p,
                  void *stream);
/* fftend (src/fft.f90:210-246): releases the plan and its device memory */
int cans_plan_destroy(cans_plan *plan);
/* device bytes held by the plan (work space + factorisations) */
long long cans_plan_device_bytes(const cans_plan *plan);
/* profiling aid (the reference's src/timer.f90 role): when enabled, CUDA events are
 * recorded on the plan's stream between the five passes of every solve (x-forward,
 * y-forward, z-elimination, y-backward, x-backward); cans_plan_get_timing synchronises
 * the stream and returns the mean milliseconds per pass over the recorded solves
 * (at most 256 since the last call) and clears them. */
int cans_plan_set_timing(cans_plan *plan, int enable);
int cans_plan_get_timing(cans_plan *plan, double ms[5], int *nsolves);
/* mean ms of the residual launches of cans_solver_refined recorded while timing is enabled
 * (count of them in *count); synchronises the plan's stream */
int cans_plan_get_residual_timing(cans_plan *plan, double *ms, int *count);
/* running total of CUDA kernel launches issued by this library in this process */
long long cans_launch_count(void);

/* ---- the Poisson / Helmholtz solve ------------------------------------------------------- */
/* solver / solver_gpu (src/solver.f90:17, src/solver_gpu.f90:34): in-place solve on
 * the interior of the haloed device field p (FP64).  Ghost cells are not touched. */
int cans_solver(cans_plan *plan, double *p);
/* same solve on an FP32 field (plan created with CANS_FP32) */
int cans_solver_f32(cans_plan *plan, float *p);
/* FP64 solve on an FP32-arithmetic plan recovered to FP64 accuracy by iterative
 * refinement: r = rhs - L p in FP64, correction solved in FP32, p += e (FP64).
 * Stops when ||r||_2 <= rtol*||rhs||_2 or after max_iter corrections; returns the
 * number of corrections in *iters and the last evaluated relative residual in *relres
 * (both may be NULL).  When the iteration ends at max_iter, the last correction is
 * added to p by its own x-backward pass and its residual is not evaluated (saves one
 * residual pass), so *relres is the residual before that correction; max_iter = 0 is one
 * FP32 solve written to p (*relres = 1).  dzci/dzfi: device grid arrays (0..n3+1). */
int cans_solver_refined(cans_plan *plan, double *p, const double dli[3], const double *dzci,
                        const double *dzfi, double rtol, int max_iter, int *iters, double *relres);
/* solve_helmholtz (src/solve_helmholtz.f90:28): p/alpha + lap(p) = rhs, 3D variant.
 * Adds the boundary RHS (updt_rhs_b with alpha) then solves with b+1/alpha and
 * normfft/alpha.  Factorisations for recent alpha values are cached in the plan. */
int cans_solve_helmholtz(cans_plan *plan, double alpha, const int is_bound[6], double *p);

/* ---- projection and momentum kernels (FP64) ---------------------------------------------- */
/* fillps (src/fillps.f90:13) */
int cans_fillps(const int n[3], const double dli[3], const double *dzfi, double dti,
                const double *u, const double *v, const double *w, double *p, void *stream);
/* correc (src/correc.f90:13) */
int cans_correc(const int n[3], const double dli[3], const double *dzci, double dt,
                const double *p, double *u, double *v, double *w, void *stream);
/* updatep (src/updatep.f90:14); is_impdiff selects p += pp + alpha*lap(pp) */
int cans_updatep(const int n[3], const double dli[3], const double *dzci, const double *dzfi,
                 double alpha, int is_impdiff, const double *pp, double *p, void *stream);
/* rk (src/rk.f90:24) with mom_xyz_ad (src/mom.f90:771): one low-storage RK3 substep of
 * the momentum equations (explicit pressure gradient, constant-flow-rate forcing).
 * dudtrko..: halo-free (n1,n2,n3) device arrays (previous substep RHS, updated).
 * work: device scratch of at least cans_rk_work_doubles(n, is_impdiff) doubles, or NULL
 * to use a scratch buffer the library allocates on first use and keeps (one per device,
 * shared by every call that passes NULL: calls that may overlap on the GPU, from other
 * streams or host threads, pass their own work).
 * f[3] (host out): the bulk-velocity forcing applied (velf - mean).  The forcing
 * reduction is done on the device; the call synchronises `stream` once when any
 * is_forced is set. */
int cans_rk(const double rkpar[2], const int n[3], const double dli[3], const double *dzci,
            const double *dzfi, const double *grid_vol_ratio_c, const double *grid_vol_ratio_f,
            double dt, double visc, const double *p, const int is_forced[3], const double velf[3],
            const double bforce[3], int is_impdiff, double *dudtrko, double *dvdtrko, double *dwdtrko,
            double *u, double *v, double *w, double f[3], double *work, void *stream);
size_t cans_rk_work_doubles(const int n[3], int is_impdiff);
/* rk with the Boussinesq buoyancy of the first scalar (src/rk.f90:24-25, gacc/beta):
 * u -= f12 * gacc * beta * (s interpolated to the face), same arguments as cans_rk plus
 * gacc[3], beta and the haloed device scalar s */
int cans_rk_buoy(const double rkpar[2], const int n[3], const double dli[3], const double *dzci,
                 const double *dzfi, const double *grid_vol_ratio_c, const double *grid_vol_ratio_f,
                 double dt, double visc, const double *p, const int is_forced[3], const double velf[3],
                 const double bforce[3], int is_impdiff, const double gacc[3], double beta, const double *s,
                 double *dudtrko, double *dvdtrko, double *dwdtrko, double *u, double *v, double *w,
                 double f[3], double *work, void *stream);
/* rk_scal (src/rk.f90:335-491) with scal (src/scal.f90:41-193): one RK3 substep of a
 * cell-centred scalar s (haloed) with diffusivity alpha, source ssource, RHS history
 * dsdtrko (halo-free); with is_impdiff the implicit part is left for the Helmholtz solve
 * (s -= f12/2 * dsdtd).  *f (host) = scalf - bulk mean when is_forced (synchronises the
 * stream), else 0.  work: cans_rk_scal_work_doubles(n, is_impdiff) device doubles. */
int cans_rk_scal(const double rkpar[2], const int n[3], const double dli[3], const double *dzci,
                 const double *dzfi, const double *grid_vol_ratio_f, double alpha, double dt,
                 const double *u, const double *v, const double *w, int is_forced, double scalf,
                 double ssource, int is_impdiff, double *dsdtrko, double *s, double *f, double *work,
                 void *stream);
size_t cans_rk_scal_work_doubles(const int n[3], int is_impdiff);
/* bulk_forcing_s (src/scal.f90:301): s += f on the interior when is_forced */
int cans_bulk_forcing_s(const int n[3], int is_forced, double f, double *s, void *stream);
/* ---- the FP32 run ------------------------------------------------------------------------
 * The routines above with FP32 fields u, v, w, p and FP32 device grid arrays (dzci, dzfi,
 * grid_vol_ratio), the form of the reference's single-precision build (src/types.f90:12-18,
 * rp = sp) except that the pressure correction pp stays FP64: it is the right-hand side and
 * solution of the FP64-accurate refined solve (cans_solver_refined on a CANS_FP32 plan).
 * Arithmetic per cell is the FP64 routines' in FP32, in the same order; global sums add
 * per-warp FP32 partial sums in FP64.  Explicit diffusion only (is_impdiff != 0 returns
 * CANS_ENOTSUP). */
/* fillps (src/fillps.f90:13): FP32 divergence of u, v, w written to the FP64 p */
int cans_fillps_f32(const int n[3], const double dli[3], const float *dzfi, double dti,
                    const float *u, const float *v, const float *w, double *p, void *stream);
/* correc (src/correc.f90:13): gradient of the FP64 p (differences of hi/lo float pairs) */
int cans_correc_f32(const int n[3], const double dli[3], const float *dzci, double dt,
                    const double *p, float *u, float *v, float *w, void *stream);
/* updatep (src/updatep.f90:14), explicit form: p += pp rounded to FP32 */
int cans_updatep_f32(const int n[3], const double dli[3], const float *dzci, const float *dzfi,
                     double alpha, int is_impdiff, const double *pp, float *p, void *stream);
/* correc (src/correc.f90:13) and the explicit updatep (src/updatep.f90:14) in one pass over
 * pp: the two read the same pp and write disjoint fields, so the host may call this in place
 * of correc, bounduvw, updatep (src/main.f90:469-471), followed by bounduvw and boundp */
int cans_correc_updatep_f32(const int n[3], const double dli[3], const float *dzci, double dt,
                            const double *pp, float *u, float *v, float *w, float *p, void *stream);
/* rk (src/rk.f90:24) with mom_xyz_ad (src/mom.f90:771): out of place when unew != u (the new
 * velocity goes to the interior of the haloed unew, vnew, wnew -- a second velocity buffer the
 * caller swaps with u, v, w afterwards; its ghost cells are left for the following bounduvw),
 * in place when unew == u, vnew == v, wnew == w.  dudtrko..: FP32 halo-free.  work: device
 * scratch of cans_rk_f32_work_bytes(n, in_place) bytes.  f[3] (host): the forcing velf - mean
 * (FP64 means); synchronises `stream` when any is_forced is set. */
int cans_rk_f32(const double rkpar[2], const int n[3], const double dli[3], const float *dzci,
                const float *dzfi, const float *grid_vol_ratio_c, const float *grid_vol_ratio_f,
                double dt, double visc, const float *p, const int is_forced[3], const double velf[3],
                const double bforce[3], int is_impdiff, float *dudtrko, float *dvdtrko, float *dwdtrko,
                float *u, float *v, float *w, float *unew, float *vnew, float *wnew, double f[3],
                void *work, void *stream);
size_t cans_rk_f32_work_bytes(const int n[3], int in_place);
/* bounduvw / boundp (src/bound.f90:17,124) on FP32 fields (same arguments) */
int cans_bounduvw_f32(const char cbc[18], const int n[3], const double bc[18], const int is_bound[6],
                      const double dl[3], const double *dzc, const double *dzf, float *u, float *v,
                      float *w, int keep_norm, int halos_norm, int halos_tang, void *stream);
int cans_boundp_f32(const char cbc[6], const int n[3], const double bc[6], const int is_bound[6],
                    const double dl[3], const double *dzc, float *p, int halo_side, void *stream);
/* chkdiv / chkdt / bulk_mean (src/chkdiv.f90:15, src/chkdt.f90:16, src/utils.f90:15) on FP32
 * fields; FP32 per-cell arithmetic, FP64 sums; synchronise `stream` */
int cans_chkdiv_f32(const int n[3], const double l[3], const double dli[3], const float *dzfi,
                    const float *u, const float *v, const float *w, double *divtot, double *divmax,
                    void *stream);
int cans_chkdt_f32(const int n[3], const double dl[3], const float *dzci, const float *dzfi,
                   double visc, double alpha, int is_impdiff, int is_impdiff_1d, const float *u,
                   const float *v, const float *w, double *dtmax, void *stream);
int cans_bulk_mean_f32(const int n[3], const float *grid_vol_ratio, const float *p, double *mean,
                       void *stream);

/* bounduvw (src/bound.f90:17), one GPU: halos_* are -1 lower, 0 none, 1 upper, 2 both
 * (argument absent in the reference).  dl: host; dzc, dzf: HOST arrays 0..n3+1
 * (only dzc(0), dzc(n3), dzf(0), dzf(n3) are read). */
int cans_bounduvw(const char cbc[18], const int n[3], const double bc[18], const int is_bound[6],
                  const double dl[3], const double *dzc, const double *dzf, double *u, double *v,
                  double *w, int keep_norm, int halos_norm, int halos_tang, void *stream);
/* boundp (src/bound.f90:124) */
int cans_boundp(const char cbc[6], const int n[3], const double bc[6], const int is_bound[6],
                const double dl[3], const double *dzc, double *p, int halo_side, void *stream);
/* updt_rhs_b (src/bound.f90:514): rhsb[6] constant face values (from cans_initsolver);
 * has_alpha = 0 when the reference's optional alpha is absent */
int cans_updt_rhs_b(const char c_or_f[3], const char cbc[6], const int n[3], const int is_bound[6],
                    const double rhsb[6], double *p, double alpha, int has_alpha, void *stream);
/* chkdiv (src/chkdiv.f90:15): device FP64 reduction, synchronises `stream`.  Returns
 * CANS_ENONFINITE (with both outputs written) when divtot or divmax is not finite -- the
 * reference's NaN test of src/main.f90:504.  cans_chkdiv, cans_chkdt and cans_bulk_mean use
 * one library-owned scratch buffer per device behind a lock, so calls from several host
 * threads are safe; they serialise. */
int cans_chkdiv(const int n[3], const double l[3], const double dli[3], const double *dzfi,
                const double *u, const double *v, const double *w, double *divtot, double *divmax,
                void *stream);
/* Divergence check that allocates nothing.  No counterpart in the reference: it is
 * cans_chkdiv with its scratch moved into a fixed device array inside the library, for
 * callers that cannot call cudaMalloc -- e.g. a Fortran host whose device memory is owned
 * by the OpenACC runtime's pool, or a long run that fixes its memory budget up front.
 * Limit: n1*n2*n3 <= 16,777,216 interior cells (65,536 blocks of 256 threads); larger sizes
 * return CANS_EINVAL and launch nothing.  The array (1 MiB) is held on every device that
 * loads the library until the process exits.  The first call on each device looks up the
 * array's device address (cudaGetSymbolAddress) with that device current; make that first
 * call before any stream capture.  All calls share the one array and it keeps the last
 * call's contents (each call writes every slot it reads), so calls that overlap on the GPU
 * (different streams or host threads at the same time) race: serialise them.  Like
 * cans_chkdiv, the call copies the two results to the host and synchronises `stream`
 * before it returns; results and arguments are those of cans_chkdiv. */
int cans_chkdiv_noalloc(const int n[3], const double l[3], const double dli[3], const double *dzfi,
                        const double *u, const double *v, const double *w, double *divtot,
                        double *divmax, void *stream);
/* chkdt (src/chkdt.f90:16): device reduction, synchronises `stream`.  dlmin is computed
 * from dl and the device dzfi as the reference does. */
int cans_chkdt(const int n[3], const double dl[3], const double *dzci, const double *dzfi,
               double visc, double alpha, int is_impdiff, int is_impdiff_1d, const double *u,
               const double *v, const double *w, double *dtmax, void *stream);
/* bulk_mean (src/utils.f90:15): device FP64 reduction, synchronises `stream` */
int cans_bulk_mean(const int n[3], const double *grid_vol_ratio, const double *p, double *mean,
                   void *stream);

/* ---------------------------------------------------------------- profile statistics
 * Plane/line averages of the output routines (device arrays in and out, asynchronous on
 * `stream`); the host writes the files.
 * cans_out1d: out1d (src/output.f90:56-157), the profile of p along idir (1..3) averaged over
 *   the other two directions; out holds n[idir-1] values; dz (device, indices 0..n3+1, the
 *   dzf or dzc array of the variable) weights the z sums of idir = 1, 2 and may be NULL for 3.
 * cans_out1d_chan: out1d_chan (src/output.f90:327-393), idir = 3 only (1 and 2 compute
 *   nothing, as in the reference): out = [um, vm, wm, u2, v2, w2, uw], n3 values each, the
 *   second moments minus the products of the means.
 * cans_out2d_duct: out2d_duct (src/output.f90:395-529), averages along the streamwise
 *   direction idir = 1 (out = [um, vm, wm, u2, v2, w2, uv, uw], each (n2, n3), j fastest) or
 *   idir = 2 (out = [um, vm, wm, u2, v2, w2, vw, uv], each (n1, n3), i fastest); idir = 3
 *   computes nothing, as in the reference. */
int cans_out1d(const int n[3], const double l[3], const double dl[3], int idir, const double *dz, const double *p,
               double *out, void *stream);
int cans_out1d_chan(const int n[3], const double l[3], const double dl[3], int idir, const double *u,
                    const double *v, const double *w, double *out, void *stream);
int cans_out2d_duct(const int n[3], const double l[3], const double dl[3], int idir, const double *u,
                    const double *v, const double *w, double *out, void *stream);

/* ---------------------------------------------------------------- checkpoints
 * load_one (src/load.f90:461-589) with the MPI-IO file layout on one rank: the file holds
 * the n1*n2*n3 interior values of the haloed device field p in Fortran order (FP64,
 * native byte order) followed by [time, istep] as two FP64 values (main.f90 names them
 * fld_u.bin, fld_v.bin, fld_w.bin, fld_p.bin).  Both synchronise `stream`.
 * cans_load_field returns CANS_EINVAL for a file whose size is not (n1*n2*n3 + 2) * 8
 * bytes (the reference aborts the run), CANS_EIO when the file cannot be opened or read;
 * ghost cells of p are left untouched (the caller applies bounduvw/boundp, main.f90:389). */
int cans_save_field(const char *path, const int n[3], const double *p, double time, int istep,
                    void *stream);
int cans_load_field(const char *path, const int n[3], double *p, double *time, int *istep,
                    void *stream);

/* ---------------------------------------------------------------- adjoints
 * No counterpart in the reference.  Transposed (vector-Jacobian) products of the FP64
 * substep routines with explicit diffusion and no flow-rate forcing, for reverse-mode
 * gradients.  Every adjoint argument g* is a device array laid out like the forward
 * quantity it belongs to; "+=" arguments accumulate. */
/* S^T g for the plan's solve S (cans_solver): g <- D^-1 S D g with D the diagonal of the
 * z operator's symmetric factorisation (dzfi, or dzci for face-centred z); in place */
int cans_solver_adjoint(cans_plan *plan, double *g);
/* the same for the linear part of cans_solve_helmholtz (no boundary terms) */
int cans_solve_helmholtz_adjoint(cans_plan *plan, double alpha, double *g);
/* fillps^T: gu, gv, gw (haloed) += D^T gp (gp interior) */
int cans_fillps_adjoint(const int n[3], const double dli[3], const double *dzfi, double dti,
                        const double *gp, double *gu, double *gv, double *gw, void *stream);
/* correc^T: gp (haloed) += G^T (gu, gv, gw); the velocity adjoints pass through */
int cans_correc_adjoint(const int n[3], const double dli[3], const double *dzci, double dt,
                        const double *gu, const double *gv, const double *gw, double *gp,
                        void *stream);
/* updatep^T (same arguments as cans_updatep): explicit (p += pp): gpp += gp on the interior;
 * is_impdiff (p += pp + alpha lap(pp), src/updatep.f90): gpp += (I + alpha lap)^T gp, which
 * also reaches the ghost cells of gpp that lap read (folded back by cans_boundp_adjoint) */
int cans_updatep_adjoint(const int n[3], const double dli[3], const double *dzci, const double *dzfi,
                         double alpha, int is_impdiff, const double *gp, double *gpp, void *stream);
/* transposes of bounduvw / boundp (same arguments): ghost adjoints go back to the
 * interior cells the ghosts were filled from, in reverse order, and are zeroed */
int cans_bounduvw_adjoint(const char cbc[18], const int n[3], const double bc[18],
                          const int is_bound[6], const double dl[3], const double *dzc,
                          const double *dzf, double *gu, double *gv, double *gw, int keep_norm,
                          int halos_norm, int halos_tang, void *stream);
int cans_boundp_adjoint(const char cbc[6], const int n[3], const double bc[6],
                        const int is_bound[6], const double dl[3], const double *dzc, double *gp,
                        int halo_side, void *stream);
/* rk^T (src/rk.f90:24 with mom_xyz_ad, explicit diffusion, is_forced = 0).  u, v, w: the
 * velocity rk read (haloed).  In: gu, gv, gw = adjoint of the velocity after rk (haloed),
 * gdu, gdv, gdw = adjoint of the dudtrko rk wrote.  Out, in place: the adjoints of the
 * input velocity and of the input dudtrko; gp (haloed) += the pressure's; gbf[3] (host,
 * may be NULL) += the uniform body force's (synchronises the stream).  work: device
 * scratch of cans_rk_adjoint_work_doubles(n) doubles. */
int cans_rk_adjoint(const double rkpar[2], const int n[3], const double dli[3], const double *dzci,
                    const double *dzfi, double dt, double visc, int is_impdiff, const double *u,
                    const double *v, const double *w, double *gu, double *gv, double *gw, double *gdu,
                    double *gdv, double *gdw, double *gp, double gbf[3], double *work, void *stream);
size_t cans_rk_adjoint_work_doubles(const int n[3]);

/* ---------------------------------------------------------------- batched solves
 * No counterpart in the reference (one box per run there).  A batch groups FP64 plans of
 * independent systems -- boxes of uneven size, and per box e.g. the three velocity
 * Helmholtz plans or the pressure plan -- and solves all of them with one persistent
 * launch per pass (x-forward, y-forward, z, y-backward, x-backward) over the
 * concatenated work of every system.  Each system uses its own plan's spectral buffer
 * and factorisations, so a plan may appear in one batch once and must not be used on
 * another stream while the batch runs. */
typedef struct cans_batch cans_batch;

/* Autotuner (no counterpart in the reference; cuFFT/FFTW choose their own plans there):
 * times the plan's x and y transform kernels for each candidate shape -- the compile-time
 * kernel of power-of-two lengths, and the generic kernel over radix orders x lines per CTA
 * -- and keeps the fastest in the plan.  Results are remembered per (precision, direction,
 * length, kinds) for the process, so plans sharing a transform are measured once, on the
 * first one tuned (force != 0 measures again).  Only the order of the transform's floating-point operations changes.
 * ms[2] (optional): the chosen x and y forward-pass times.  Synchronises the plan's
 * stream; not allowed during stream capture. */
int cans_plan_autotune(cans_plan *plan, int force, double ms[2]);
/* current shape of direction d (0 x, 1 y): radix order, lines per CTA, compile-time length
 * (0: generic kernel) */
int cans_plan_get_shape(const cans_plan *plan, int d, int radix[12], int *nstages, int *ncx,
                        int *spec);
/* Non-finite check of the plan's solves (the reference tests only the divergence for NaN,
 * src/main.f90:503-509): every z pass records whether its spectral data held a NaN or Inf
 * (a non-finite right-hand side value reaches all of it).  Synchronises the plan's stream;
 * returns CANS_ENONFINITE when a solve since the last check saw one, CANS_ETIMEOUT when a
 * bounded wait of the TMA-tiled z pass expired (its results are then not valid), CANS_OK
 * otherwise; clears the record. */
int cans_plan_check(cans_plan *plan);
/* Self-test of the bounded device waits (no counterpart in the reference): launches one CTA
 * that waits on an mbarrier nothing arrives on, with a limit of limit_us microseconds
 * (1..100000); *expired = 1 when the wait gave up and the kernel returned normally, as the
 * tiled z pass's waits do before reporting CANS_ETIMEOUT.  Synchronises the device. */
int cans_selftest_wait_timeout(int limit_us, int *expired);
/* z pass of an FP32 plan (no counterpart in the reference; the elimination of
 * src/solver_gpu.f90:278-428): mode 0 = one thread per spectral column sweeping all rows with
 * precomputed factors; 1 = the column split into 16-row segments held in registers, factors
 * formed on the fly, the segments joined by a cyclic reduction of their separator rows (non-
 * periodic z with at most 512 rows); 2 = tiles of 32 columns x all rows moved into shared
 * memory by TMA (each value read and written once), factors formed on the fly, up to 16
 * segments per column joined by a cyclic reduction that also closes periodic z (n1 n2 a
 * multiple of 4, at most 512 rows); -1 = the automatic choice (mode 2 where it applies; the
 * default).  CANS_ENOTSUP for a mode the plan's shape does not allow (and for FP64 plans,
 * which have mode 0 only).  cans_plan_autotune measures the available modes and keeps the
 * fastest.  Results differ between the modes only by FP32 rounding. */
int cans_plan_set_zpass(cans_plan *plan, int mode);
int cans_plan_get_zpass(const cans_plan *plan, int *mode);
int cans_batch_create(int nsys, cans_plan *const *plans, void *stream, cans_batch **batch);
int cans_batch_destroy(cans_batch *batch);
/* System s, on the field p[s] (device, haloed):
 *   alpha[s] != 0: cans_solve_helmholtz(plans[s], alpha[s], is_bound + 6*s, p[s])
 *                  (src/solve_helmholtz.f90:28-75);
 *   alpha[s] == 0: cans_updt_rhs_b(c_or_f, cbc, n, is_bound + 6*s, rhsb, p[s], 1, 0)
 *                  followed by cans_solver(plans[s], p[s]) (src/bound.f90:514,
 *                  src/solver_gpu.f90:34).
 * alpha == NULL: every system is a Poisson solve; is_bound == NULL: no boundary terms.
 * Results are bit-identical to those single calls.  The boundary terms are added while
 * the x-forward pass loads the field (p itself is then overwritten by the solution).
 * The first call with a given (p, alpha, is_bound) builds and caches a device work table
 * (and the factorisations for new alphas); later calls with the same arguments launch
 * the five pass kernels only, and may be captured into a CUDA graph.  A call during
 * stream capture whose table is not cached returns CANS_ENOTSUP. */
int cans_batch_solve(cans_batch *batch, double *const *p, const double *alpha,
                     const int *is_bound);

/* ---------------------------------------------------------------- batched boxes
 * No counterpart in the reference.  Many independent boxes (e.g. closed boxes / lid-driven
 * cavities of uneven size), each with its own grid, BCs, viscosity and fixed time step,
 * advanced together: every stage of an RK3 substep (rk + mom, the velocity Helmholtz
 * solves, bounduvw, fillps, updt_rhs_b + pressure solve, boundp, correc, updatep) is one
 * persistent launch over all boxes, and a time step can be captured once as a CUDA graph.
 * Each box evolves bit-identically to the single-box call sequence of src/main.f90:452-472
 * with a fixed dt (dt_f) and no flow-rate forcing.  The caller owns the fields. */
typedef struct cans_box {
  int n[3];              /* interior cells */
  double l[3];           /* domain lengths: dl = l/n, dli = 1/dl */
  double visc, dt;       /* 1/Re and the fixed time step */
  char cbcvel[18];       /* cbcvel(0:1,3,3) order */
  char cbcpre[6];
  double bcvel[18], bcpre[6], bforce[3];
  const double *dzc_g, *dzf_g;  /* host z grid (0:n3+1), as cans_initgrid returns */
  const double *dzci, *dzfi;    /* device 1/dzc, 1/dzf (0:n3+1) */
  double *u, *v, *w, *p, *pp;   /* device haloed fields (n1+2)(n2+2)(n3+2) */
  double *dudtrko, *dvdtrko, *dwdtrko;  /* device n1*n2*n3 */
} cans_box;
typedef struct cans_boxes cans_boxes;
/* builds per box the pressure plan (and, when is_impdiff, the three velocity Helmholtz
 * plans: c_or_f 'f' along the component), the device work lists of every stage and two
 * solve batches; allocates 3 (6 with is_impdiff) doubles per cell of scratch */
int cans_boxes_create(int nbox, const cans_box *boxes, int is_impdiff, int autotune,
                      void *stream, cans_boxes **out);
int cans_boxes_destroy(cans_boxes *boxes);
/* bounduvw + boundp on the initial fields (src/main.f90:388-418) */
int cans_boxes_start(cans_boxes *boxes);
/* RK3 substep irk (0, 1, 2) of every box, asynchronous on the stream */
int cans_boxes_substep(cans_boxes *boxes, int irk);
/* one time step (three substeps).  use_graph != 0: the first call runs the step and
 * captures it as a CUDA graph (needs a non-default stream); later calls replay the graph */
int cans_boxes_step(cans_boxes *boxes, int use_graph);
/* kernel nodes of the captured step graph (0 before capture) */
long long cans_boxes_graph_nodes(const cans_boxes *boxes);

#ifdef __cplusplus
}
#endif
#endif
