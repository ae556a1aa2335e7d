/* Layout of the C ABI structs and values of its constants, as the C compiler
 * sees include/muscade_gpu.h: one line per struct ("S name size") and per field
 * ("F struct field offset"), and per constant ("C name value"). */
#include <stddef.h>
#include <stdio.h>

#include "muscade_gpu.h"

#define S(T) printf("S %s %zu\n", #T, sizeof(T))
#define F(T, f) printf("F %s %s %zu\n", #T, #f, offsetof(T, f))
#define C(N) printf("C %s %ld\n", #N, (long)(N))

int main(void) {
  S(mgpu_group);
  F(mgpu_group, kind), F(mgpu_group, nX), F(mgpu_group, nU), F(mgpu_group, ndata), F(mgpu_group, nele);
  F(mgpu_group, indexX), F(mgpu_group, indexU), F(mgpu_group, edata), F(mgpu_group, indexA);
  S(mgpu_model_desc);
  F(mgpu_model_desc, nX), F(mgpu_model_desc, nU), F(mgpu_model_desc, ngroup), F(mgpu_model_desc, groups);
  F(mgpu_model_desc, scaleX), F(mgpu_model_desc, device), F(mgpu_model_desc, nA);
  S(mgpu_newmark);
  F(mgpu_newmark, a1), F(mgpu_newmark, a2), F(mgpu_newmark, a3), F(mgpu_newmark, b1), F(mgpu_newmark, b2);
  F(mgpu_newmark, b3);
  S(mgpu_sweep_opts);
  F(mgpu_sweep_opts, beta), F(mgpu_sweep_opts, gamma), F(mgpu_sweep_opts, maxiter), F(mgpu_sweep_opts, maxdx);
  F(mgpu_sweep_opts, maxLl), F(mgpu_sweep_opts, fixed_iter), F(mgpu_sweep_opts, per_component);
  F(mgpu_sweep_opts, no_graph), F(mgpu_sweep_opts, device_loop);
  S(mgpu_stats);
  F(mgpu_stats, nstep_done), F(mgpu_stats, niter_total), F(mgpu_stats, fail_step), F(mgpu_stats, fail_iter);
  F(mgpu_stats, last_dx), F(mgpu_stats, last_Ll);
  S(mgpu_linsolve_info);
  F(mgpu_linsolve_info, kind), F(mgpu_linsolve_info, ncomp), F(mgpu_linsolve_info, max_kl);
  F(mgpu_linsolve_info, max_ku), F(mgpu_linsolve_info, last_fallback), F(mgpu_linsolve_info, last_sweeps);
  S(mgpu_tune_report);
  F(mgpu_tune_report, elem_block), F(mgpu_tune_report, linsolve), F(mgpu_tune_report, ms_elem);
  F(mgpu_tune_report, ms_linsolve);
  S(mgpu_sparse_report);
  F(mgpu_sparse_report, nfront), F(mgpu_sparse_report, nheight), F(mgpu_sparse_report, nroot);
  F(mgpu_sparse_report, max_front), F(mgpu_sparse_report, max_pivots), F(mgpu_sparse_report, fp64);
  F(mgpu_sparse_report, front_entries), F(mgpu_sparse_report, flops), F(mgpu_sparse_report, last_fallback);
  F(mgpu_sparse_report, last_sweeps), F(mgpu_sparse_report, last_perturbed), F(mgpu_sparse_report, last_factor_ms);
  F(mgpu_sparse_report, last_refine_ms);
  C(MGPU_OK), C(MGPU_ERR_ARG), C(MGPU_ERR_CUDA), C(MGPU_ERR_UNSUPPORTED), C(MGPU_ERR_NAN), C(MGPU_ERR_SINGULAR);
  C(MGPU_ERR_NOCONV), C(MGPU_ERR_NOMEM), C(MGPU_ERR_SIZE);
  C(MGPU_EULERBEAM3D), C(MGPU_BAR3D), C(MGPU_DOFCONSTRAINT_X), C(MGPU_DOFLOAD);
  C(MGPU_DOFCOST), C(MGPU_SINGLEUDOF), C(MGPU_ACOST);
  C(MGPU_ASM_STATIC), C(MGPU_ASM_STEP), C(MGPU_ASM_ITER);
  C(MGPU_LINSOLVE_AUTO), C(MGPU_LINSOLVE_F32IR), C(MGPU_LINSOLVE_F64), C(MGPU_LINSOLVE_BLOCK);
  C(MGPU_LINSOLVE_TORN), C(MGPU_LINSOLVE_TORN32), C(MGPU_LINSOLVE_SPARSE), C(MGPU_LINSOLVE_SPARSE64);
  return 0;
}
