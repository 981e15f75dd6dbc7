/*
 * CPU oracle for the CaNS pressure-correction path -- TEST INFRASTRUCTURE ONLY.
 *
 * A plain C99 (+OpenMP) restatement of the reference's CPU algorithms, used
 * by tests/ to check the CUDA path, by __graft_entry__.smoke() and by
 * bench.py's cpu_baseline / reference arm.  Nothing in the product library
 * (cans_gb300/) links, loads or calls this code.
 *
 * Parity pin: a full 1500-step replay of the reference's lid-driven-cavity
 * regression case (tests/lid_driven_cavity/{input.nml,data_ldc_re1000.txt})
 * is checked against the reference's own golden v-profile at rtol 1e-7, and
 * every r2r kind is checked against scipy.fft (pocketfft) and direct O(N^2)
 * sums (tests/test_oracle_*.py).
 *
 * Conventions (Fortran layout, as the reference):
 *   - 3D fields carry one ghost layer: extents (n1+2, n2+2, n3+2), i fastest,
 *     element (i,j,k) with 0 <= i <= n1+1 at  i + (n1+2)*(j + (n2+2)*k).
 *   - 1D grid arrays dzc, dzf, dzci, dzfi, zc, zf are indexed 0..n3+1.
 *   - boundary-condition characters cbc(0:1,3) are passed as 6 chars,
 *     cbc[ibound + 2*idir]; velocity cbcvel(0:1,3,3) as 18 chars,
 *     cbcvel[ibound + 2*idir + 6*icomp]; values bc/bcvel likewise.
 */
#ifndef CANS_ORACLE_H
#define CANS_ORACLE_H
#include <stddef.h>
#ifdef __cplusplus
extern "C" {
#endif

/* FFTW r2r kind ids, as src/fftw.f90:62-85 */
enum { ORC_R2HC = 0, ORC_HC2R = 1, ORC_REDFT00 = 3, ORC_REDFT01 = 4, ORC_REDFT10 = 5,
       ORC_REDFT11 = 6, ORC_RODFT00 = 7, ORC_RODFT01 = 8, ORC_RODFT10 = 9, ORC_RODFT11 = 10 };

int  orc_num_threads(void);
void orc_set_num_threads(int n);

/* src/initgrid.f90:14-99 (+ gridpoint_* 105-175); gtype 1..4 */
int orc_initgrid(int gtype, int n, double gr, double lz, int is_periodic,
                 double *dzc, double *dzf, double *zc, double *zf);
/* src/initsolver.f90:85-144 (CPU ordering, no GPU reorder) */
void orc_eigenvalues(int n, const char bc[2], char c_or_f, double *lambda);
/* src/initsolver.f90:146-187 */
void orc_tridmatrix(const char bc[2], int n, const double *dzci, const double *dzfi, char c_or_f,
                    double *a, double *b, double *c);
/* src/fft.f90:260-313 */
void orc_find_fft(const char bc[2], char c_or_f, int *kind_fwd, int *kind_bwd, double norm[2]);
/* src/initsolver.f90:15-83 + fft.f90:25-209 (normfft part).  Outputs:
 *   lambdaxy[n1*n2] (i fastest), a,b,c[n3], *normfft,
 *   rhsb[6] = constant face values rhsb{x,y,z}(:,:,0:1) -> rhsb[ibound + 2*idir] */
void orc_initsolver(const int ng[3], const double dli[3], const double *dzci_g, const double *dzfi_g,
                    const char cbc[6], const double bc[6], const char c_or_f[3],
                    double *lambdaxy, double *a, double *b, double *c, double *normfft, double rhsb[6]);

/* one FFTW-semantics r2r transform of length n on `howmany` lines:
 * element m of line l sits at data[l*dist + m*stride] (FFTW guru r2r, unnormalised) */
int orc_r2r(int kind, int n, long howmany, long stride, long dist, double *data);
/* r2r along x (dir 0) or y (dir 1) of a halo-free (nx,ny,nz) array, on the first nt points */
int orc_r2r_dir(int kind, int dir, int nt, int nx, int ny, int nz, double *data);

/* src/solver.f90:114-307, p halo-free (nx,ny,n_p) with n_p >= n (+1 if periodic uses n rows);
 * lambdaxy may be NULL */
void orc_gaussel(int nx, int ny, int n, int ldz, const double *a, const double *b, const double *c,
                 int is_periodic, double norm, double *p, const double *lambdaxy);
/* src/solver.f90:17-112: one Poisson/Helmholtz solve, in place on haloed p */
int orc_solver(const int n[3], double normfft, const double *lambdaxy, const double *a,
               const double *b, const double *c, const char cbc[6], const char c_or_f[3], double *p);
/* src/solve_helmholtz.f90:28-75 (3D variant) */
int orc_solve_helmholtz(const int n[3], double normfft, double alpha, const double *lambdaxy,
                        const double *a, const double *b, const double *c, const double rhsb[6],
                        const int is_bound[6], const char cbc[6], const char c_or_f[3], double *p);

/* src/fillps.f90:13-51 */
void orc_fillps(const int n[3], const double dli[3], const double *dzfi, double dti,
                const double *u, const double *v, const double *w, double *p);
/* src/correc.f90:13-60 */
void orc_correc(const int n[3], const double dli[3], const double *dzci, double dt,
                const double *p, double *u, double *v, double *w);
/* src/updatep.f90:14-88 (is_impdiff selects the implicit branch) */
void orc_updatep(const int n[3], const double dli[3], const double *dzci, const double *dzfi,
                 double alpha, int is_impdiff, const double *pp, double *p);
/* src/mom.f90:771-1019 (fused advection-diffusion); dudtd may be NULL when !is_impdiff.
 * dudt/dudtd are halo-free (n1,n2,n3). */
void orc_mom_xyz_ad(const int n[3], double dxi, double dyi, const double *dzci, const double *dzfi,
                    double visc, const double *u, const double *v, const double *w,
                    double *dudt, double *dvdt, double *dwdt, double *dudtd, double *dvdtd, double *dwdtd,
                    int is_impdiff);
/* src/utils.f90:15-42 */
double orc_bulk_mean(const int n[3], const double *grid_vol_ratio, const double *p);
/* src/rk.f90:24-333 (no scalars/buoyancy; mom_xyz_ad fast path).  dudtrko: halo-free.
 * work: 6*n1*n2*n3 doubles scratch.  f[3] out. */
void orc_rk(const double rkpar[2], const int n[3], const double dli[3], const double *dzci,
            const double *dzfi, const double *gvr_c, const double *gvr_f, double dt, double visc,
            const double *p, const int is_forced[3], const double velf[3], const double bforce[3],
            int is_impdiff, double *dudtrko, double *dvdtrko, double *dwdtrko,
            double *u, double *v, double *w, double f[3], double *work);
void orc_rk_buoy(const double rkpar[2], const int n[3], const double dli[3], const double *dzci,
                 const double *dzfi, const double *gvr_c, const double *gvr_f, double dt, double visc,
                 const double *p, const int is_forced[3], const double velf[3], const double bforce[3],
                 int is_impdiff, const double gacc[3], double beta, const double *sb, double *dudtrko,
                 double *dvdtrko, double *dwdtrko, double *u, double *v, double *w, double f[3], double *work);
void orc_scal(const int n[3], double dxi, double dyi, const double *dzci, const double *dzfi, double alpha,
              const double *u, const double *v, const double *w, const double *s, double *dsdt, double *dsdtd,
              int is_impdiff);
double orc_rk_scal(const double rkpar[2], const int n[3], const double dli[3], const double *dzci,
                   const double *dzfi, const double *gvr_f, double alpha, double dt, const double *u,
                   const double *v, const double *w, int is_forced, double scalf, double ssource, int is_impdiff,
                   double *dsdtrko, double *s, double *work);
void orc_bulk_forcing_s(const int n[3], int is_forced, double f, double *s);
/* src/bound.f90:17-122 (CPU path, one rank, x-aligned pencils) */
void orc_bounduvw(const char cbc[18], const int n[3], const double bc[18], const int is_bound[6],
                  const double dl[3], const double *dzc, const double *dzf,
                  double *u, double *v, double *w, int keep_norm, int halos_norm, int halos_tang);
/* src/bound.f90:124-180 */
void orc_boundp(const char cbc[6], const int n[3], const double bc[6], const int is_bound[6],
                const double dl[3], const double *dzc, double *p, int halo_side);
/* src/bound.f90:514-598, rhsb as constants per face */
void orc_updt_rhs_b(const char c_or_f[3], const char cbc[6], const int n[3], const int is_bound[6],
                    const double rhsb[6], double *p, double alpha, int has_alpha);
/* src/chkdt.f90:16-78 */
double orc_chkdt(const int n[3], const double dl[3], const double *dzci, const double *dzfi,
                 double visc, double alpha, int is_impdiff, int is_impdiff_1d,
                 const double *u, const double *v, const double *w);
/* src/chkdiv.f90:15-54 */
void orc_chkdiv(const int n[3], const double l[3], const double dli[3], const double *dzfi,
                const double *u, const double *v, const double *w, double *divtot, double *divmax);

/* r = rhs - L x in long double for the cell-centred Poisson operator the solver inverts
 * (x/y second differences with P/N/D ghosts, z rows a, b, c); r halo-free */
void orc_poisson_residual_ld(const int n[3], const double dli[3], const char cbc[6], const double *a,
                             const double *b, const double *c, const double *x, const double *rhs, double *r);

/* seeded uniform noise (this project's generator, NOT gfortran's random_number):
 * p(i,j,k) += 2*(r-0.5)*norm over the interior, r = splitmix64 of (seed, global index) */
void orc_add_noise(const int n[3], unsigned long long seed, double norm, double *p);

/* initflow (src/initflow.f90:16-259), one rank: interiors of u, v, w, p (HOST grid arrays
 * 0..n3+1); noise from orc_add_noise (seeds 123, 456, 789).  -1 for an unknown case. */
int orc_initflow(const char *inivel, const double bcvel[18], const int n[3], const double l[3], const double dl[3],
                 const double *zc, const double *zf, const double *dzc, const double *dzf, double visc,
                 const int is_forced[3], const double velf[3], const double bforce[3], int is_wallturb, double *u,
                 double *v, double *w, double *p);
/* its 1D profile part: 1 for the 3D analytic cases (tgv, tgw, ant), -1 unknown */
int orc_initflow_profile(const char *inivel, const double bcvel[18], int n3, const double l[3], const double *zc,
                         double visc, const int is_forced[3], const double velf[3], const double bforce[3],
                         int is_wallturb, double *u1d, double *ubulk, int *is_noise, int *is_mean);

/* ---------- whole-run driver (src/main.f90:144-520, single rank, no I/O) ---------- */
/* profile statistics of src/output.f90 (out1d 56-157, out1d_chan 327-393, out2d_duct 395-529) */
void orc_out1d(const int n[3], const double l[3], const double dl[3], int idir, const double *dz, const double *p,
               double *out);
void orc_out1d_chan(const int n[3], const double l[3], const double dl[3], const double *u, const double *v,
                    const double *w, double *out);
void orc_out2d_duct(const int n[3], const double l[3], const double dl[3], int idir, const double *u,
                    const double *v, const double *w, double *out);

typedef struct orc_case {
  int ng[3];
  double l[3];
  int gtype; double gr;
  double cfl, dtmax, dt_f, visci;
  int icheck;
  char cbcvel[18]; double bcvel[18];
  char cbcpre[6];  double bcpre[6];
  double bforce[3]; int is_forced[3]; double velf[3];
  int is_impdiff;
  /* one transported scalar when nscal = 1 (&scalar of src/param.f90:144-151) */
  int nscal;
  double alphai; char cbcscal[6]; double bcscal[6]; double ssource; int is_sforced; double scalf;
  double gacc[3]; double beta; int is_buoyancy;
} orc_case;

typedef struct orc_state orc_state;
/* setup: grid, solver(s), allocations; fields start at zero */
orc_state *orc_state_new(const orc_case *cs);
void orc_state_free(orc_state *s);
/* raw pointers into the state: which = 0 u,1 v,2 w,3 p,4 pp,5 scalar (haloed),
 * 10 dzc,11 dzf,12 zc,13 zf,14 dzci,15 dzfi (0..n3+1), 20 lambdaxy_p, 21 ap,22 bp,23 cp */
double *orc_state_ptr(orc_state *s, int which);
/* boundary conditions + initial dt (main.f90:388-418); call after fields are set */
void orc_state_start(orc_state *s);
/* one full time step (3 RK substeps + dt/divergence check when istep % icheck == 0) */
void orc_state_step(orc_state *s);
/* scalars: 0 time, 1 dt, 2 istep, 3 divtot, 4 divmax, 5..7 dpdl, 8 normfft_p, 9 fs (scalar forcing) */
double orc_state_scalar(orc_state *s, int which);

#ifdef __cplusplus
}
#endif
#endif
