// FP32 solve recovered to FP64 accuracy by iterative refinement (placeholder until the
// refinement kernels land).
#include "cans_internal.cuh"

extern "C" int cans_solver_refined(cans_plan *plan, double *p, const double dli[3], const double *dzci,
                                   const double *dzfi, double rtol, int max_iter, int *iters, double *relres) {
  (void)plan; (void)p; (void)dli; (void)dzci; (void)dzfi; (void)rtol; (void)max_iter; (void)iters; (void)relres;
  return CANS_ENOTSUP;
}
