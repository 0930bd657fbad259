// Batched PCG over many independent problems (batching form).
#include "gbpa_internal.cuh"

extern "C" int gbpa_batched_pcg_solve(gbpa_ctx_t ctx, int nprob, const gbpa_problem_desc *probs,
                                      double rel_tol, double abs_tol, int max_it, int *iterations,
                                      int *converged, double *final_norms, double *seconds)
{
   (void)ctx; (void)nprob; (void)probs; (void)rel_tol; (void)abs_tol; (void)max_it;
   (void)iterations; (void)converged; (void)final_norms; (void)seconds;
   return GBPA_ERR_UNSUPPORTED;
}
