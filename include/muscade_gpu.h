/*
 * muscade_gpu.h -- C ABI of the GB300 assemble-and-solve path for Muscade.jl
 * models built from EulerBeam3D, Bar3D, Hold / DofConstraint{:X} (affine gap,
 * equal mode), DofLoad and the quadratic cost elements SingleDofCost,
 * SingleUdof and SingleAcost.
 *
 * The Julia side keeps Model / addelement! / initialize! and the element API;
 * it hands the device what its Disassembler already holds (per element type,
 * the model dof indices of each element and the element objects' fields) and
 * calls these entry points from a new solver type, SweepXGPU{OX}, that
 * `solve` dispatches to beside SweepX (src/Solve.jl:16-35).
 *
 * Conventions
 *   - Dof indices are 1-based Int64, exactly `dis.dis[ieletyp].index[iele].X`
 *     (src/Assemble.jl:22-99), laid out [nele][nX] row-major.
 *   - Vectors and matrices are Float64; sparse matrices are CSC with 1-based
 *     colptr/rowval like SparseMatrixCSC.
 *   - Host buffers are owned by the caller; the context owns device memory
 *     and its CUDA stream.  A context is not re-entrant: one per host thread.
 *   - Every call returns MGPU_OK (0) or an error code; mgpu_last_error()
 *     gives the message.  No call falls back to the CPU.
 */
#ifndef MUSCADE_GPU_H
#define MUSCADE_GPU_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* status codes; messages follow the reference's muscadeerror texts */
#define MGPU_OK 0
#define MGPU_ERR_ARG 1          /* invalid argument or layout */
#define MGPU_ERR_CUDA 2         /* CUDA runtime / library failure */
#define MGPU_ERR_UNSUPPORTED 3  /* element kind the GPU path does not support */
#define MGPU_ERR_NAN 4          /* "residual(...) returned NaN in R, FB or derivatives" (src/Assemble.jl:625) */
#define MGPU_ERR_SINGULAR 5     /* "matrix factorization failed at step=..., iiter=..." (src/SweepX.jl:209) */
#define MGPU_ERR_NOCONV 6       /* "no convergence of step ... after ... iterations" (src/SweepX.jl:221) */
#define MGPU_ERR_NOMEM 7        /* device allocation failed */
#define MGPU_ERR_SIZE 8         /* problem larger than a fixed-capacity entry point allows */

/* element kinds */
#define MGPU_EULERBEAM3D 1     /* toolbox/BeamElement.jl:87-208; nX=12 (+nU=3 when udof); edata: 69 fields */
#define MGPU_BAR3D 2           /* toolbox/BarElement.jl:89-202; nX=6 (+nU=3); edata: 38 fields */
#define MGPU_DOFCONSTRAINT_X 3 /* src/BasicElements.jl:406-438,484-488; nX=nx+1; edata: nx gap coefficients */
#define MGPU_DOFLOAD 4         /* src/BasicElements.jl:275-284; nX=1; no edata */
/* Cost elements, with the quadratic cost functor cost(v, t) = w (v − y(t))²
 * whose target y(t) is a time value evaluated by the caller like a load:
 *   MGPU_DOFCOST     SingleDofCost of class :X (src/BasicElements.jl:32-50,198-208):
 *                    L = w (x⁽ᵈ⁾ − y(t))² on one X-dof; nX=1; edata: w, d (0, 1 or 2,
 *                    the time derivative); one time value y(t).  In SweepX
 *                    R = ∂L/∂Λ = 0.
 *   MGPU_SINGLEUDOF  SingleUdof (src/BasicElements.jl:239-248): L = w (u − y(t))² − λu
 *                    with λ the X-dof's multiplier; nX=1, nU=1; edata: w; one time
 *                    value y(t).  In SweepX R = −u on the X-dof (the U-dof's value
 *                    is a load).
 *   MGPU_ACOST       SingleAcost (src/BasicElements.jl:77-86,163-167): the once-off
 *                    L = w (a − y)² on one A-dof; nX=0, indexA; edata: w, y. */
#define MGPU_DOFCOST 5
#define MGPU_SINGLEUDOF 6
#define MGPU_ACOST 7

/* One element type (one entry of model.eleobj / dis.dis). */
typedef struct {
  int32_t kind;          /* MGPU_EULERBEAM3D ... */
  int32_t nX;            /* X-dofs per element */
  int32_t nU;            /* U-dofs per element (0 or 3 for beams/bars) */
  int32_t ndata;         /* doubles per element in edata */
  int64_t nele;          /* number of elements */
  const int64_t *indexX; /* [nele][nX] 1-based model X-dof indices */
  const int64_t *indexU; /* [nele][nU] 1-based model U-dof indices (NULL if nU==0) */
  const double *edata;   /* [nele][ndata] element fields in the reference's declaration order */
  const int64_t *indexA; /* [nele] 1-based A-dof of each element, NULL if none.  EULERBEAM3D:
                            the EI scale factor of the wrapper element EulerBeam3D{adof}
                            (bending stiffnesses EI2, EI3 times the A-dof value); ACOST:
                            the A-dof of the cost (required) */
} mgpu_group;

typedef struct {
  int64_t nX;               /* getndof(model,:X) */
  int64_t nU;               /* getndof(model,:U) */
  int32_t ngroup;           /* number of element types, in model order */
  const mgpu_group *groups; /* [ngroup] */
  const double *scaleX;     /* [nX] dof scales (dis.scaleX), NULL for all ones */
  int32_t device;           /* CUDA device ordinal */
  int64_t nA;               /* getndof(model,:A) */
} mgpu_model_desc;

/* Newmark-β coefficients (src/SweepX.jl:3-15) */
typedef struct {
  double a1, a2, a3, b1, b2, b3;
} mgpu_newmark;

/* missions of one assembly (src/SweepX.jl:39-96) */
#define MGPU_ASM_STATIC 0  /* SweepX{0}: Lλ = R, Lλx = K                      */
#define MGPU_ASM_STEP 1    /* SweepX{2} first iteration: Lλ = R - C a - M b, Lλx = K + a1 C + b1 M */
#define MGPU_ASM_ITER 2    /* SweepX{2} later iterations: Lλ = R, Lλx = K + a1 C + b1 M */

typedef struct mgpu_ctx mgpu_ctx;

/* Build the device model: CSC pattern and element-entry maps (replaces
 * prepare(AssemblySweepX), src/SweepX.jl:24-33 with asmvec!/asmmat!,
 * src/Assemble.jl:340-448), upload element data and dof maps. */
int mgpu_create(mgpu_ctx **ctx, const mgpu_model_desc *desc);
void mgpu_destroy(mgpu_ctx *ctx);
const char *mgpu_last_error(const mgpu_ctx *ctx);

/* Sparsity of Lλx: nnz, then colptr[nX+1] and rowval[nnz] (1-based), and the
 * asm maps of element type `igroup`: asm1[nele][nX] (position in Lλ) and
 * asm2[nele][nX*nX] (position in nzval, entry i+nX*j), as asm[1|2,ieletyp]
 * (src/Assemble.jl:340-448). */
int64_t mgpu_nnz(const mgpu_ctx *ctx);
int mgpu_get_pattern(const mgpu_ctx *ctx, int64_t *colptr, int64_t *rowval);
int mgpu_get_asm(const mgpu_ctx *ctx, int32_t igroup, int64_t *asm1, int64_t *asm2);

/* Number of time-dependent element values per assembly: one per DofLoad
 * element (F(t)), one per DofConstraint element (gap offset c(t) in
 * g = Σ aᵢxᵢ − c(t)) and one per DOFCOST or SINGLEUDOF element (the cost
 * target y(t)), concatenated over groups in model order. */
int64_t mgpu_ntval(const mgpu_ctx *ctx);

/* Kernel launches enqueued so far by the context's assembly, Newton and
 * multifrontal paths (the banded solvers' kernels are not counted); the
 * difference over a region counts the launches inside it. */
int64_t mgpu_launch_count(const mgpu_ctx *ctx);

/* One assembly with host buffers (replaces assemble!{:step|:iter} over the
 * AssemblySweepX elements, src/Assemble.jl:470-505 with addin!, src/SweepX.jl:39-96).
 *   x[nXder][nX] (X, X', X''), u[nU], tvals[ntval] at time t.
 *   Outputs (host, may be NULL): Ll[nX] (Lλ) and nzval[nnz] (Lλx.nzval). */
int mgpu_assemble(mgpu_ctx *ctx, int32_t mission, int32_t nXder, const double *x, const double *u, double t,
                  const double *tvals, const mgpu_newmark *c, double *Ll, double *nzval);

/* The same assembly, pipelined: enqueues it and returns a ticket.  The inputs
 * are copied before the call returns (the caller may reuse x, u, tvals at
 * once).  Ll and nzval receive the outputs by the time mgpu_assemble_wait
 * returns for that ticket; until then the caller must leave them alone.  At
 * most two assemblies are in flight: a third call first waits for the copies
 * of the oldest.  The outputs of one call are copied back while the next one
 * computes, so a loop of calls costs the larger of the two, not their sum.
 * mgpu_assemble_wait takes one of the last two tickets and reports a NaN in
 * that assembly with the same message as mgpu_assemble. */
int mgpu_assemble_async(mgpu_ctx *ctx, int32_t mission, int32_t nXder, const double *x, const double *u, double t,
                        const double *tvals, const mgpu_newmark *c, double *Ll, double *nzval, int64_t *ticket);
int mgpu_assemble_wait(mgpu_ctx *ctx, int64_t ticket);

/* Element-level evaluation like diffed_residual (src/Diagnostic.jl:929-965)
 * for the elements of group `igroup`:  X[nele][nXder][nX], U[nele][nU].
 * Returns R[nele][nX] and, per element, dR[nele][nX][nX] (column-major per
 * element: ∂R_i/∂ with respect to p0·X₀ + p1·X₁ + p2·X₂ in direction j at
 * i + nX*j) and, when U is given and dRdU != NULL, dRdU[nele][nX][nU]. */
int mgpu_element_eval(mgpu_ctx *ctx, int32_t igroup, int32_t nXder, const double *X, const double *U, double t,
                      double p0, double p1, double p2, double *R, double *dR, double *dRdU);

/* Element-level Lagrangian like diffed_lagrangian{2} (src/Diagnostic.jl:852-927)
 * for the elements of group `igroup` of kind DOFLOAD or DOFCONSTRAINT_X
 * (residual elements, L = Λ·R), DOFCOST, SINGLEUDOF or ACOST: the value and
 * the first and second derivatives over the element's variables in the order
 * DirectXUA revariates them (src/DirectXUA.jl:152-171) and adds them into its
 * per-step gradient and Hessian blocks (:122-151):
 *   Λ[nX], X⁽⁰⁾[nX], .., X⁽ⁿˣᵈᵉʳ⁻¹⁾[nX], U[nU], A[nA]
 * so np = nX (1 + nXder) + nU + nA (nA = 1 for ACOST, else 0).  Inputs per
 * element: lam[nele][nX], X[nele][nXder][nX], U[nele][nU], A[nele][nA] and
 * tv[nele], the group's time values at the evaluation time (F, c or y; unused
 * by ACOST, whose target is in edata).  Outputs (each may be NULL): L[nele],
 * dL[nele][np], d2L[nele][np][np] (symmetric).  A DOFCOST on X⁽ᵈ⁾ needs
 * nXder > d.  EulerBeam3D and Bar3D (residual elements without second order)
 * return MGPU_ERR_UNSUPPORTED: use mgpu_element_eval. */
int mgpu_element_lagrangian(mgpu_ctx *ctx, int32_t igroup, int32_t nXder, const double *lam, const double *X,
                            const double *U, const double *A, const double *tv, double *L, double *dL, double *d2L);

/* Element results of the EulerBeam3D group `igroup`, like getresult
 * (src/Output.jl:131-181) of the values its residual makes requestable
 * (toolbox/BeamElement.jl:151-189): for each of nstate states X[nstate][nX]
 * and each element, 50 values: ε, rₛₘ (9, column-major), then per Gauss point
 * (4) x (3), κ (3), fᵢ = EA ε and mᵢ = (GJ κ₁, EI₃ κ₂, EI₂ κ₃) (the EI scale
 * of an A-dof applied).  out[nstate][nele][50]. */
int mgpu_beam_results(mgpu_ctx *ctx, int32_t igroup, int64_t nstate, const double *X, double *out);

/* Device-resident assembly for throughput measurement: upload a state once,
 * then assemble repeatedly into device buffers.  mgpu_time_assemble runs
 * `reps` assemblies timed with CUDA events on the context stream (optionally
 * writing a 512 MB buffer before each, to flush the L2) and reports the mean
 * device time of the whole assembly, of each element type's kernel
 * (ms_groups[ngroup], may be NULL) and of the two scatter kernels. */
int mgpu_upload_state(mgpu_ctx *ctx, int32_t nXder, const double *x, const double *u, const double *tvals);
int mgpu_assemble_resident(mgpu_ctx *ctx, int32_t mission, double t, const mgpu_newmark *c);
int mgpu_download(mgpu_ctx *ctx, double *Ll, double *nzval);
int mgpu_time_assemble(mgpu_ctx *ctx, int32_t mission, double t, const mgpu_newmark *c, int32_t reps,
                       int32_t flush_l2, double *ms_total, double *ms_groups, double *ms_scatter);

/* Solver options (keywords of solve(SweepX{OX}), src/SweepX.jl:179-184) */
typedef struct {
  double beta, gamma; /* Newmark-β parameters (OX=2) */
  int32_t maxiter;    /* maximum Newton iterations per step */
  double maxdx;       /* convergence: Σ Δx² ≤ maxdx² */
  double maxLl;       /* and Σ Lλ² ≤ maxLl² (use +Inf to disable) */
  int32_t fixed_iter; /* > 0: exactly this many iterations per step, no convergence test
                         (the reference has no such option; used for fixed-cost time stepping).
                         The steps then replay one captured CUDA graph (up to 63 iterations) and
                         the host waits for the device only at the end of the sweep. */
  int32_t per_component; /* != 0: the convergence test is applied to each connected component
                            of Lλx on its own (independent models solved together); a component
                            that passes stops iterating while the others go on, so each follows
                            the iterations it would take alone.  Needs fixed_iter = 0. */
  int32_t no_graph;      /* != 0: fixed-iteration steps are launched kernel by kernel */
  int32_t device_loop;   /* != 0 (SweepX{0}, banded FP64 or F32IR solver, convergence test): the whole
                            sweep is one CUDA graph launch whose conditional WHILE nodes loop over the
                            load steps and the Newton iterations on the device (per-component test with
                            per_component), bounded by maxiter; the host reads nothing until it ends */
} mgpu_sweep_opts;

typedef struct {
  int32_t nstep_done;  /* steps that converged (states written) */
  int32_t niter_total; /* Newton iterations over all steps */
  int32_t fail_step;   /* 1-based step of a failure, else 0 */
  int32_t fail_iter;   /* 1-based iteration of a failure, else 0 */
  double last_dx;      /* √ΣΔx² of the last iteration */
  double last_Ll;      /* √ΣLλ² of the last iteration */
} mgpu_stats;

/* Whole SweepX{OX} solve on the device (src/SweepX.jl:179-226), OX ∈ {0,2}.
 *   times[nstep], t0 = initial state time, x0[nXder0][nX] initial X and
 *   derivatives (nXder0 ≤ OX+1; missing derivatives are zero), u[nU],
 *   tvals[nstep][ntval].  states[nstep][OX+1][nX] receives the converged X
 *   (and X', X'') of every step; on error the steps before the failing one
 *   are written and stats->nstep_done tells how many. */
int mgpu_sweepx(mgpu_ctx *ctx, int32_t OX, int64_t nstep, const double *times, double t0, int32_t nXder0,
                const double *x0, const double *u, const double *tvals, const mgpu_sweep_opts *opts, double *states,
                mgpu_stats *stats);

/* Values of the A-dofs, A[nA] (initially all 1: the nominal EI).  Copied; in
 * effect for the following assemblies and solves. */
int mgpu_set_A(mgpu_ctx *ctx, const double *A);

/* Cost sensitivities of a SweepX{OX} run by the discrete adjoint (the
 * analogue of DirectXUA's ∂C/∂A, src/DirectXUA.jl:438-513, for the Newmark
 * time discretisation).  Runs the converged forward sweep (fixed_iter = 0,
 * per_component = 0; opts as for mgpu_sweepx), keeping the state at the start
 * of every segment of `ckpt` steps (ckpt <= 0: ⌈√nstep⌉), then walks the steps
 * backwards, recomputing each segment from its checkpoint, and solves the
 * transposed tangent of every step.  The cost is the Lagrangian of the
 * model's cost elements plus optional sensor arrays:
 *   C = Σ_n w_n [ Σ_DOFCOST w_e (x_n⁽ᵈᵉ⁾[i_e] − y_e(t_n))² + Σ_SINGLEUDOF w_e (u[j_e] − y_e(t_n))²
 *               + Σ_s cost_w[s] (x_n[cost_dof[s]] − cost_y[n][s])² ]  +  Σ_ACOST w_e (a[k_e] − y_e)²
 * with w_n = t_n − t_{n−1} for OX = 2 (t_0 = t0) and 1 for OX = 0 (DirectXUA
 * weighs its steps alike), the targets y_e(t_n) taken from tvals, the A-costs
 * counted once, and cost_dof[ncost] distinct 1-based X-dofs (ncost may be 0).
 * Outputs: *cost, dCdA[nA] (EI-scale and A-cost A-dofs); when dCdtv != NULL,
 * dCdtv[nstep][ntval]: the sensitivities to the load values F(t) of DofLoad
 * elements, the gap offsets c(t) of DofConstraint elements and the cost
 * targets y(t), in the layout of tvals; when dCdU != NULL, dCdU[nU]: the
 * sensitivities to the U-dofs of SINGLEUDOF elements, held through the sweep
 * as SweepX holds U (MGPU_ERR_UNSUPPORTED if a beam or bar has U-dofs).
 * A DOFCOST on X' or X'' needs OX = 2.  Needs the row-band solver for the
 * transposed tangent. */
int mgpu_adjoint_sweepx(mgpu_ctx *ctx, int32_t OX, int64_t nstep, const double *times, double t0, int32_t nXder0,
                        const double *x0, const double *u, const double *tvals, const mgpu_sweep_opts *opts,
                        int64_t ncost, const int64_t *cost_dof, const double *cost_w, const double *cost_y,
                        int32_t ckpt, double *cost, double *dCdA, double *dCdtv, double *dCdU, mgpu_stats *stats);

/* Forward sensitivities of a SweepX{OX} run with respect to a few A-dofs (the
 * forward-mode counterpart of mgpu_adjoint_sweepx; SweepXA assembles the same
 * sensitivity system, src/SweepXA.jl:49-221).  Runs the converged forward
 * sweep and, after every step, solves the step's tangent once per selected
 * A-dof θ:  Jₙ sₓ = −∂R/∂θ − Cₙ gᵥ − Mₙ gₐ  (gᵥ, gₐ the parts of X′, X″ carried
 * from the previous step's sensitivities), sᵥ = a1 sₓ + gᵥ, sₐ = b1 sₓ + gₐ.
 * sel[nsel] are distinct 1-based A-dofs; the cost is that of
 * mgpu_adjoint_sweepx (cost elements plus optional sensor arrays).  Outputs
 * (each may be NULL): dXdA[nstep][nsel][OX+1][nX], the sensitivities of X (and
 * X′, X″); dCdA[nsel], the cost gradient at the selected A-dofs. */
int mgpu_sensitivity_sweepx(mgpu_ctx *ctx, int32_t OX, int64_t nstep, const double *times, double t0,
                            int32_t nXder0, const double *x0, const double *u, const double *tvals,
                            const mgpu_sweep_opts *opts, int64_t ncost, const int64_t *cost_dof, const double *cost_w,
                            const double *cost_y, int32_t nsel, const int64_t *sel, double *dXdA, double *dCdA,
                            mgpu_stats *stats);

/* Linear solver of the Newton loops (no counterpart in the reference, which
 * calls UMFPACK through lu/lu!/\ at src/SweepX.jl:207-210).  Every connected
 * component of Lλx is reordered (reverse Cuthill-McKee) and factorised as a
 * band with partial pivoting:
 *   MGPU_LINSOLVE_AUTO   TORN32 when some component has 512 dofs or more and
 *                        max(kl, ku) <= 16 -- switching to TORN for the rest of
 *                        the context's life after the first solve that needs the
 *                        FP64 fallback -- else F64 where every component has
 *                        kl <= 31 and kl+ku+1 <= 64, else BLOCK (the default)
 *   MGPU_LINSOLVE_F32IR  FP32 factors, FP64 residuals and iterative refinement
 *                        until the correction is below 1e-12 of the solution;
 *                        a component that does not contract, or would need
 *                        more than 8 sweeps, is refactorised in FP64
 *   MGPU_LINSOLVE_F64    FP64 factors, one warp per component
 *   MGPU_LINSOLVE_BLOCK  FP64 factors, one thread block per component, bands up to 256
 *   MGPU_LINSOLVE_TORN   FP64, long components cut into about √(n/s) interiors
 *                        factorised in parallel and separators of s = max(kl, ku)
 *                        dofs coupled through their banded Schur complement
 *                        (pivoting within each interior and within the Schur band)
 *   MGPU_LINSOLVE_TORN32 the partitioned factorisation in FP32 inside 4 sweeps of
 *                        FP64 iterative refinement; a component whose last
 *                        correction is not below 1e-10 of its solution is solved
 *                        again with the FP64 partitioned factorisation
 *   MGPU_LINSOLVE_SPARSE multifrontal LU for matrices whose bands are too wide
 *                        (3D frames, lattices; AUTO picks it there): groups of
 *                        dofs with equal couplings (the dofs of a node, a Hold's
 *                        multiplier with the dof it holds) ordered by nested
 *                        dissection of the element geometry, fronts of dense
 *                        blocks factorised without row exchanges (multipliers
 *                        after the dofs they constrain) on the equilibrated
 *                        matrix, FP32 factors inside FP64 iterative refinement
 *                        until the scaled correction is below 1e-14 of the
 *                        scaled solution or stops shrinking below 1e-10 of it
 *                        (at most 12 sweeps), else the FP64 factors, which then
 *                        stay in use for the context
 *   MGPU_LINSOLVE_SPARSE64 the multifrontal LU in FP64 throughout
 * F64 and BLOCK give bitwise the same Δx.  Returns MGPU_ERR_UNSUPPORTED when
 * the bands are too wide for the requested kind.  The multifrontal kinds
 * need fixed_iter steps without graph replay and no per_component test, and
 * give no transposed solve (mgpu_adjoint_sweepx). */
#define MGPU_LINSOLVE_AUTO 0
#define MGPU_LINSOLVE_F32IR 1
#define MGPU_LINSOLVE_F64 2
#define MGPU_LINSOLVE_BLOCK 3
#define MGPU_LINSOLVE_TORN 4
#define MGPU_LINSOLVE_TORN32 5
#define MGPU_LINSOLVE_SPARSE 6
#define MGPU_LINSOLVE_SPARSE64 7
int mgpu_set_linear_solver(mgpu_ctx *ctx, int32_t kind);

typedef struct {
  int32_t kind;          /* MGPU_LINSOLVE_F32IR, _F64, _BLOCK, _TORN, _TORN32, _SPARSE or _SPARSE64 in use */
  int32_t ncomp;         /* connected components of Lλx */
  int32_t max_kl;        /* widest lower / upper band after reordering (multifrontal: the largest front) */
  int32_t max_ku;
  int32_t last_fallback; /* F32IR, TORN32: components refactorised in FP64 in the last solve */
  int32_t last_sweeps;   /* F32IR, TORN32: refinement sweeps in the last solve */
} mgpu_linsolve_info;
int mgpu_linear_solver_info(mgpu_ctx *ctx, mgpu_linsolve_info *info);

/* The multifrontal solver's structure and its last solve (no counterpart in
 * the reference).  MGPU_ERR_UNSUPPORTED when the model has none. */
typedef struct {
  int32_t nfront;         /* fronts (supernodes) */
  int32_t nheight;        /* levels of the elimination tree, leaves at 0 */
  int32_t nroot;          /* independent trees (connected components) */
  int32_t max_front;      /* largest front (dofs) */
  int32_t max_pivots;     /* most pivots of one front */
  int32_t fp64;           /* 1 when factorising in FP64 */
  int64_t front_entries;  /* entries of all fronts (the factor storage) */
  double flops;           /* flops of one factorisation (2 per multiply-add) */
  int32_t last_fallback;  /* 1 when the last solve fell back to FP64 factors */
  int32_t last_sweeps;    /* refinement sweeps of the last solve */
  int32_t last_perturbed; /* FP32 pivots below 1e-10 set to ±1e-10 in the last factorisation */
  double last_factor_ms;  /* device time of the last solve's factorisation(s) (CUDA events) */
  double last_refine_ms;  /* and of its substitutions and refinement sweeps */
} mgpu_sparse_report;
int mgpu_sparse_info(mgpu_ctx *ctx, mgpu_sparse_report *rep);

/* Autotuner (no counterpart in the reference): on the resident state (after
 * mgpu_upload_state) times one assembly of `mission` with 64, 128 and 256
 * threads per block of the element kernels, and then the factorisation and
 * solve of the assembled matrix with every applicable linear solver kind, and
 * keeps the fastest of each for the following assemblies and solves.  Timings
 * are means of 3 runs after one warm-up, CUDA events on the context stream. */
typedef struct {
  int32_t elem_block;     /* chosen threads per block */
  int32_t linsolve;       /* chosen MGPU_LINSOLVE_* */
  double ms_elem[3];      /* assembly with 64, 128, 256 threads per block */
  double ms_linsolve[6];  /* factorisation + solve by MGPU_LINSOLVE_* index, < 0 when not applicable */
} mgpu_tune_report;
int mgpu_autotune(mgpu_ctx *ctx, int32_t mission, const mgpu_newmark *c, mgpu_tune_report *rep);

/* Beam assembly that allocates nothing (no counterpart in the reference).
 * For callers that cannot call cudaMalloc where they assemble -- inside a
 * captured CUDA graph, in a loop whose device memory was fixed beforehand, or
 * when device memory belongs to another runtime's pool.  Every argument is
 * device memory the caller owns:
 *   fields[nele][69]   EulerBeam3D fields (as mgpu_group.edata)
 *   indexX[nele][12]   1-based model X-dofs of each beam
 *   asm1[nele][12]     1-based positions in Lλ      (asm[1,ieletyp], 0 = skip)
 *   asm2[nele][144]    1-based positions in nzval   (asm[2,ieletyp], 0 = skip)
 *   x[nX]              state X
 *   Ll[nX], nzval[nnz] outputs, overwritten (zeroed, then summed)
 * It computes the SweepX{0} residual and tangent of the beams and enqueues
 * the work on `stream` (a cudaStream_t, NULL for the legacy stream) without
 * synchronising.  For beams without U- or A-dofs and with unit dof scales the
 * results equal those of mgpu_assemble with MGPU_ASM_STATIC on a model of
 * these beams; U-dof loads, A-dof EI scales and dis.scaleX are not applied.
 * No NaN check is made: a NaN in an element shows in Ll / nzval, which the
 * caller reads.  A CUDA error already pending on the calling thread is
 * returned as MGPU_ERR_CUDA before anything is enqueued.  Its scratch is one
 * fixed device array that every GPU loading the library holds until exit, so
 * nele is limited to MGPU_NOALLOC_MAX_BEAMS (returns MGPU_ERR_SIZE above it).
 * All calls on a device share that array: calls that overlap on the GPU
 * (different streams, or host threads without ordering) race and must be
 * serialised by the caller.  The first call on each device looks up the
 * array's device address (cudaGetSymbolAddress) with that device current and
 * keeps it for the life of the process; make that first call before any
 * stream capture, and do not call this entry point again after
 * cudaDeviceReset on that device (the kept address belongs to the old
 * context). */
#define MGPU_NOALLOC_MAX_BEAMS 4096
int mgpu_assemble_beams_noalloc(int64_t nele, int64_t nX, int64_t nnz, const double *fields, const int64_t *indexX,
                                const int64_t *asm1, const int64_t *asm2, const double *x, double *Ll,
                                double *nzval, void *stream);

/* Page-lock a caller's host buffer (cudaHostRegister) so that the copies of
 * the calls above run at full host-device bandwidth and without staging;
 * optional.  Unregister before freeing the buffer. */
int mgpu_host_register(void *ptr, int64_t bytes);
int mgpu_host_unregister(void *ptr);

/* Measurement utility (no counterpart in the reference): FP64 FMA throughput
 * of `device` in TFLOP/s, from independent DFMA chains timed with CUDA events;
 * the roofline denominator of the FP64-bound element kernels. */
int mgpu_measure_fp64_peak(int32_t device, double *tflops);

/* Tensor-core check (no counterpart in the reference): C[M×N] −= A[M×K]·B[K×N]
 * for column-major FP32 host arrays, K ≤ 4096, through the tile routine of the
 * multifrontal solver's FP32 trailing update (tcgen05 kind::tf32 MMAs, each
 * operand split into a TF32 part and an FP32 remainder, three products per
 * k-step, FP32 accumulation in tensor memory). */
int mgpu_tc_gemm_check(int32_t device, int32_t M, int32_t N, int32_t K, const float *A, const float *B, float *C);

#ifdef __cplusplus
}
#endif
#endif /* MUSCADE_GPU_H */
