/*
 * topopt_gb300.h -- C ABI of libtopopt_gb300.so, a GB300 (sm_103a) drop-in for
 * the per-design-iteration SIMP compliance loop of TopOpt.jl.
 *
 * All functions return an int status (TOG_OK = 0).  On failure the message is
 * available from tog_last_error() (thread-local).  Arrays are plain host
 * pointers unless a name ends in _dev; indices are 0-based (TopOpt.jl is
 * 1-based: a dof d there is d-1 here).  Dof-sized vectors are in the
 * reference's Ferrite dof order; element-sized vectors in the reference's cell
 * order (x fastest).  A handle owns its device memory and one CUDA stream; it
 * is not thread-safe (one handle per Julia task), as the reference solver.
 *
 * Each entry point names the TopOpt.jl interface it replaces (paths relative
 * to the TopOpt.jl project root).
 */
#ifndef TOPOPT_GB300_H
#define TOPOPT_GB300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define TOG_ABI_VERSION 1

enum tog_status {
    TOG_OK = 0,
    TOG_ERR_ARG = 1,           /* ArgumentError / DimensionMismatch in the reference */
    TOG_ERR_CUDA = 2,          /* CUDA runtime error (message in tog_last_error) */
    TOG_NOT_CONVERGED = 3,     /* PCG stopped at maxiter (the reference's cg! returns silently) */
    TOG_BREAKDOWN = 4,         /* p'Kp <= 0 or NaN: operator not positive definite */
    TOG_ERR_STATE = 5,         /* call order violated (e.g. compliance before a solve) */
    TOG_ERR_OOM = 6            /* device allocation failed */
};

enum tog_precision {
    TOG_FP64 = 0,              /* plain FP64 Jacobi PCG */
    TOG_FP32_IR = 1            /* FP32 K*u and PCG inside FP64 iterative refinement */
};

enum tog_filter_kind { TOG_FILTER_NONE = 0, TOG_FILTER_DENSITY = 1, TOG_FILTER_SENS = 2 };
/* warm_start of tog_simp_step: 0 cold, 1 previous displacement; for 3D handles with
 * tog_set_warm_start_net / tog_record_next_step buffers also TOG_WARM_LEARNED (the previous
 * displacement moved by the Galerkin step on span{network correction, last displacement
 * change}) and TOG_WARM_EXTRAPOLATE (the same step along the last change alone, the ablation
 * without the network). */
enum tog_warm_start { TOG_WARM_COLD = 0, TOG_WARM_PREVIOUS = 1, TOG_WARM_LEARNED = 2, TOG_WARM_EXTRAPOLATE = 3 };
enum tog_filter_op { TOG_FILTER_J = 0, TOG_FILTER_JT = 1 };
enum tog_projection_kind { TOG_PROJ_HEAVISIDE = 1, TOG_PROJ_SIGMOID = 2 };
enum tog_element_state { TOG_ELEM_FREE = 0, TOG_ELEM_BLACK = 1, TOG_ELEM_WHITE = 2 };
enum tog_optimizer { TOG_OPT_OC = 0, TOG_OPT_MMA = 1 };
enum tog_convergence { TOG_CONV_DEFAULT = 0, TOG_CONV_ENERGY = 1 };

typedef struct tog_handle tog_handle;

/* Problem and solver settings: PointLoadCantilever / HalfMBB grid
 * (src/TopOptProblems/problem_types.jl:162-231, 324-395), material
 * (matrices_and_vectors.jl:83-84) and FEASolver keywords xmin / penalty
 * (src/FEA/solvers_api.jl:468-489). */
typedef struct tog_problem_desc {
    int32_t dim;            /* 2 (quad4) or 3 (hex8) */
    int32_t nel[3];         /* elements per axis (nel[2] ignored in 2D) */
    double size[3];         /* element edge lengths */
    double E;               /* Young's modulus E0 */
    double nu;              /* Poisson ratio */
    int32_t plane_stress;   /* 0 = plane strain, as the reference; 1 = plane stress (2D extra) */
    double xmin;            /* rho = xmin + (1 - xmin) x^p */
    double penalty;         /* PowerPenaltyFun exponent p */
} tog_problem_desc;

typedef struct tog_solve_stats {
    int32_t status;          /* TOG_OK, TOG_NOT_CONVERGED or TOG_BREAKDOWN */
    int32_t iterations;      /* PCG iterations (sum of inner iterations for FP32-IR) */
    int32_t outer_iterations;/* refinement steps (0 for FP64) */
    int32_t reserved;
    double rel_residual;     /* ||f - K u|| / ||f|| (FP64 true residual for FP32-IR) */
    double abs_residual;
} tog_solve_stats;

typedef struct tog_iter_stats {
    double compliance;       /* c = sum rho_e u_e' Ke u_e at the filtered design */
    double volume;           /* volume fraction of the filtered design before the OC step */
    double change;           /* max |x_new - x| */
    double lambda;           /* OC multiplier */
    int32_t cg_iterations;
    int32_t outer_iterations;
    int32_t oc_steps;
    int32_t status;
    double rel_residual;
} tog_iter_stats;

/* ---- library -------------------------------------------------------------------- */
const char* tog_version(void);
const char* tog_last_error(void);
/* Number of kernels this process launched through the library (graph nodes included). */
int64_t tog_launch_count(void);

/* ---- host-only helpers (no GPU needed) ------------------------------------------ */
/* Grid sizes of RectilinearGrid (src/TopOptProblems/grids.jl:66-92). */
int tog_grid_counts(int32_t dim, const int32_t* nel, int64_t* nnodes, int64_t* ncells, int64_t* ndofs);
/* Metadata.node_dofs (src/TopOptProblems/metadata.jl:116-145): node_dofs[n*dim+c],
 * node n in the reference's node order (x fastest); 0-based dofs. */
int tog_node_dofs(int32_t dim, const int32_t* nel, int32_t* node_dofs);
/* Metadata.cell_dofs (metadata.jl:40-50): cell_dofs[e*ndpc + dim*a + c]. */
int tog_cell_dofs(int32_t dim, const int32_t* nel, int32_t* cell_dofs);
/* One element stiffness matrix Ke (matrices_and_vectors.jl:68-177), Ferrite dof order,
 * row-major ndpc x ndpc. */
int tog_element_stiffness(int32_t dim, const double* size, double E, double nu, int32_t plane_stress,
                          double* Ke);

/* ---- solver handle: FEASolver(GB300Solver, problem; xmin, penalty)
 *      (replaces FEASolver(CGMatrixFreeSolver, ...), src/FEA/solvers_api.jl:468-593) -- */
int tog_create(const tog_problem_desc* desc, tog_handle** out);
int tog_destroy(tog_handle* h);
/* Launch on the caller's stream (cudaStream_t as void*); NULL restores the handle's own. */
int tog_set_stream(tog_handle* h, void* stream);
/* problem.ch.prescribed_dofs (homogeneous Dirichlet; solvers_api.jl:515-530). */
int tog_set_fixed_dofs(tog_handle* h, int64_t n, const int32_t* dofs);
/* globalinfo.f, dense, reference dof order (matrices_and_vectors.jl:346-365). */
int tog_set_rhs(tog_handle* h, const double* f);
/* setpenalty!(solver, p) (solvers_api.jl:417-427). */
/* The PCG stop rule, FEASolver's conv keyword (src/FEA/solvers_api.jl:482):
 * TOG_CONV_DEFAULT stops on the recurrence residual norm (IterativeSolvers' default), and
 * TOG_CONV_ENERGY on EnergyCriteria (src/FEA/convergence_criteria.jl:26-45): the relative
 * change of x'Ax and |x'r| / x'Ax both <= max(rtol ||r0||, abstol), checked on the start
 * vector and after every iteration; a NaN or negative x'Ax gives TOG_BREAKDOWN (the
 * reference's DomainError).  EnergyCriteria applies to TOG_FP64 solves; TOG_FP32_IR
 * rejects it with TOG_ERR_ARG. */
int tog_set_convergence(tog_handle* h, int32_t criteria);
int tog_set_penalty(tog_handle* h, double p);
/* solver.vars .= x  (compliance.jl:65): the filtered pseudo-densities, one per cell. */
int tog_set_vars(tog_handle* h, const double* x);
/* mul!(y, ::MatrixFreeOperator, x) (matrix_free_operator.jl:66-105), FP64, reference order. */
int tog_matvec(tog_handle* h, const double* x, double* y);
/* solver() -> solve_system!(CGMatrixFreeSolver, ...) (solvers_api.jl:253-282, 177-220):
 * Jacobi PCG to ||f - K u|| <= max(rtol*||f||, abstol).  warm_start != 0 starts from the
 * current u (previous solve or tog_set_u) instead of 0. */
int tog_solve(tog_handle* h, int32_t precision, double rtol, double abstol, int32_t maxiter, int32_t warm_start,
              tog_solve_stats* stats);
/* One iteration's operator kernel of the Jacobi PCG (the inner loop of cg!,
 * solvers_api.jl:197-218, over MatrixFreeOperator mul!, matrix_free_operator.jl:66-105):
 * p = D^-1 r + beta p_old, q = K(rho) p (prescribed rows: meandiag p) and p.q, run once
 * on caller vectors (reference dof order) in TOG_FP64 or, for TOG_FP32_IR, in the FP32
 * arithmetic of the refinement's inner PCG.  pq may be NULL. */
int tog_pcg_operator(tog_handle* h, int32_t precision, double beta, const double* r, const double* p_old, double* p,
                     double* q, double* pq);
/* solver.u (reference dof order). */
int tog_get_u(tog_handle* h, double* u);
int tog_set_u(tog_handle* h, const double* u);
/* ComplianceFun call + rrule (compliance.jl:58-76, compute_element_energy.jl:18-38):
 * c = sum rho_e u_e'Ke u_e at the current vars and u; grad (may be NULL) = dc/dvars. */
int tog_compliance(tog_handle* h, double* c, double* grad);

/* ---- filters: DensityFilterFun / SensFilterFun (src/CheqFilters/density_filter.jl:25-121,
 *      sens_filter.jl:29-111, CheqFilters.jl:66-118) ---------------------------------- */
/* Build the node-based filter of radius rmin (TOG_ERR_ARG if no cell has a node within rmin,
 * as DensityFilterFun's ArgumentError). */
int tog_filter_setup(tog_handle* h, double rmin);
/* op = TOG_FILTER_J: y = J x (DensityFilterFun forward, SensFilterFun pullback);
 * op = TOG_FILTER_JT: y = J' x (DensityFilterFun pullback). Cell-sized host arrays. */
int tog_filter_apply(tog_handle* h, int32_t op, const double* in, double* out);

/* HeavisideProjectionFun / SigmoidProjectionFun (src/Utilities/penalties.jl:75-96), the
 * projections of ProjectedDensityFilterFun (src/CheqFilters/density_filter.jl:130-169):
 * y = P(x) and dydx = P'(x) elementwise on cell-sized host arrays (beta >= 0).  Shares the
 * filter's device scratch. */
int tog_projection(tog_handle* h, int32_t kind, double beta, const double* x, double* y, double* dydx);

/* ---- active-element mask: FixedElementProjectorFun (src/Functions/fixed_element.jl:13-159) ----
 * state[e] (one byte per cell, cell order) is TOG_ELEM_FREE, TOG_ELEM_BLACK (density 1) or
 * TOG_ELEM_WHITE (density 0); null makes every cell free.  A black-and-white cell cannot be
 * expressed, the reference's ArgumentError for it belongs to the caller's constructor.  With a
 * mask set, the OC update and the SIMP loop hold the fixed cells at their densities (their
 * volume counts against volfrac, as the reference's VolumeFun on the projected field). */
int tog_set_fixed_elements(tog_handle* h, const uint8_t* state);
/* count(free) (get_free_variable_count, fixed_element.jl:95); ncells without a mask */
int tog_free_variable_count(tog_handle* h, int64_t* nfree);
/* rho = p(x_free) (fixed_element.jl:44-58): black 1, white 0, free cells copied from x_free
 * in cell order.  TOG_ERR_ARG when nfree differs from the free count (the reference's
 * ArgumentError).  Host arrays: x_free of nfree entries (may be null when nfree = 0), rho
 * of ncells. */
int tog_fixed_element_project(tog_handle* h, const double* x_free, int64_t nfree, double* rho);
/* the rrule's pullback (fixed_element.jl:68-79): dx_free = drho[free]. */
int tog_fixed_element_pullback(tog_handle* h, const double* drho, double* dx_free);

/* ---- optimality-criteria update (no reference counterpart: the published OC method
 *      with move limit and eta = 1/2, bisection on lambda in [0, 1e9] to 1e-3) ---------- */
/* x_new = clamp(x sqrt(max(0,-dc)/(dv lambda)), max(0,x-move), min(1,x+move)) with
 * sum(vol_weights . x_new) = volfrac.  Cell-sized host arrays.  Cells fixed by
 * tog_set_fixed_elements keep their densities. */
int tog_oc_update(tog_handle* h, const double* x, const double* dc, const double* dv, const double* vol_weights,
                  double volfrac, double move, double* x_new, double* change, double* lambda);

/* ---- multi-load compliance: MultiLoad (src/TopOptProblems/multiload.jl:21-46) with
 *      MeanComplianceFun / BlockComplianceFun (src/Functions/mean_compliance.jl:8-150,
 *      block_compliance.jl:7-110) ----
 * The rhs columns F (CSC: colptr[ncol + 1], 0-based reference dof rows, values) are solved
 * one after the other from zero (solvers_api.jl:293-348), prescribed dofs zeroed
 * (apply_zero!), at the current vars; c[i] = f_i' u_i.  The cell gradient of every column
 * stays on the device for tog_multiload_gradient.  Precision and tolerances as tog_solve.
 * The handle's own rhs is kept; its displacement is that of the last column.  stats sums
 * the PCG iterations of all columns; TOG_NOT_CONVERGED when a column missed the tolerance. */
int tog_multiload_compliance(tog_handle* h, int32_t ncol, const int64_t* colptr, const int32_t* rowval,
                             const double* nzval, int32_t precision, double rtol, double abstol, int32_t maxiter,
                             double* c, tog_solve_stats* stats);
/* out = sum_i w[i] dc_i/dx over the columns of the last tog_multiload_compliance: the mean
 * compliance's gradient with w = 1/n, BlockComplianceFun's pullback with w = delta. */
int tog_multiload_gradient(tog_handle* h, int32_t ncol, const double* w, double* out);

/* ---- MMA, the method of moving asymptotes (Svanberg 1987), one inequality constraint ----
 * The optimizer of TopOpt.jl's SIMP scripts (Nonconvex MMA87: docs/tutorials/simp.qmd:107-114,
 * test/integration/test_end_to_end.jl:30-47), which is not part of TopOpt.jl: the published
 * method with the asymptote, bound and coefficient rules of Svanberg's 2007 notes on
 * x in [0, 1]^n, its dual solved by bisection on the multiplier.  The handle keeps the
 * asymptotes and the last two iterates between calls (tog_mma_reset starts over).
 * Minimises f subject to g(x) <= 0 given df0 = df/dx, g and dg = dg/dx at x; move is the
 * move limit (0.5 in Svanberg's notes).  Cells fixed by tog_set_fixed_elements keep their
 * densities.  Cell-sized host arrays. */
int tog_mma_update(tog_handle* h, const double* x, const double* df0, double g, const double* dg, double move,
                   double* x_new, double* change, double* lambda);
int tog_mma_reset(tog_handle* h);

/* ---- one SIMP design iteration, device-resident --------------------------------------
 * filter -> solve -> compliance/sensitivities -> filter pullback -> OC, the loop of
 * docs/tutorials/simp.qmd:86-114 with OC in place of MMA. */
/* filter_kind: TOG_FILTER_NONE / DENSITY / SENS (needs rmin > 0). x0: initial design. */
/* The optimizer of tog_simp_step: TOG_OPT_OC (default; tog_simp_init's move) or TOG_OPT_MMA
 * (volume constraint sum(w x) <= volfrac; move <= 0 selects 0.5).  Restarts MMA's history. */
int tog_simp_set_optimizer(tog_handle* h, int32_t optimizer, double move);
int tog_simp_init(tog_handle* h, int32_t filter_kind, double rmin, double volfrac, double move, const double* x0);
/* precision: TOG_FP64 (cold start, as the reference) or TOG_FP32_IR; warm_start: see
 * tog_warm_start (nonzero starts each solve from the previous displacement). */
int tog_simp_step(tog_handle* h, int32_t precision, double rtol, int32_t maxiter, int32_t warm_start,
                  tog_iter_stats* stats);
int tog_get_design(tog_handle* h, double* x);
int tog_set_design(tog_handle* h, const double* x);
/* Filtered (physical) densities of the last step. */
int tog_get_physical(tog_handle* h, double* xf);

/* ---- measurement hooks (no reference counterpart) ------------------------------------
 * Launch one solver kernel nlaunch times on the handle's stream over the handle's own PCG
 * vectors, starting from a fresh PCG state at r = f, without a host sync:
 * kernel 0 = the matrix-free PCG operator, 1 = the PCG vector update. */
int tog_bench_kernel(tog_handle* h, int32_t kernel, int32_t precision, int32_t nlaunch);
/* Algorithmic bytes moved by one launch of that kernel. */
int tog_kernel_bytes(tog_handle* h, int32_t kernel, int32_t precision, double* bytes);

/* ---- batched 2D SIMP (no counterpart in TopOpt.jl: many independent problems at once) --
 * nprob 2D cantilevers (PointLoadCantilever-style: left edge clamped, unit load [0,-1] at
 * node (nelx, load_j)), each with its own size, volume fraction and filter radius, sharing
 * the element size and material of `material` (dim 2).  Every design iteration of all
 * problems (density filter, FP32-IR solve, compliance, filter pullback, OC) is ONE CUDA
 * graph launch whose PCG and bisection loops run as device-side conditional nodes. */
typedef struct tog_batch tog_batch;
typedef struct tog_batch_stats {
    int32_t steps;           /* design iterations done */
    int32_t pcg_loops;       /* PCG iterations of the slowest problem in the last step */
    int32_t failed;          /* problems whose solve did not converge in the last step */
    int32_t reliable_updates; /* FP64 true-residual refreshes of all problems in the last step */
} tog_batch_stats;
int tog_batch_create(int32_t nprob, const int32_t* nelx, const int32_t* nely, const int32_t* load_j,
                     const double* volfrac, const double* rmin, const tog_problem_desc* material, double rtol,
                     int32_t maxiter, tog_batch** out);
int tog_batch_destroy(tog_batch* b);
int tog_batch_set_stream(tog_batch* b, void* stream);
/* Chooses the operator's band height (8, 16, 32 or 64 node rows per work item of 30 node
 * columns) and the persistent grid of the FP32 operator by timing PCG iterations of all
 * problems; re-records the graph.  Touches only solver scratch (the design and
 * displacements are unchanged). */
int tog_batch_autotune(tog_batch* b, int32_t* tile_rows);
/* Sets the band height (8, 16, 32 or 64) without timing; re-records the graph. */
int tog_batch_set_tile_rows(tog_batch* b, int32_t tile_rows);
int tog_batch_step(tog_batch* b, tog_batch_stats* stats);
/* Per-problem compliance, max design change and PCG iterations of the last step (may be NULL). */
int tog_batch_results(tog_batch* b, double* compliance, double* change, int32_t* cg_iterations);
int tog_batch_get_design(tog_batch* b, int32_t prob, double* x);
/* Per-problem solve outcome of the last step (arrays may be NULL): FP64 residual norm
 * ||f - K u|| at the last refresh, reliable updates (refreshes), status (TOG_OK converged,
 * TOG_NOT_CONVERGED failed). */
int tog_batch_solve_info(tog_batch* b, double* residual, int32_t* refreshes, int32_t* status);
/* Measurement hooks: launch one loop kernel nlaunch times over ALL problems (after the
 * set-up kernels of a design iteration, outside the graph; only solver scratch changes)
 * and return the mean microseconds per launch.  kernel 0 = FP32 operator, 1 = PCG vector
 * update, 2 = FP64 true residual, 3 = operator + update (one PCG loop). */
int tog_batch_bench_kernel(tog_batch* b, int32_t kernel, int32_t nlaunch, double* us_per_launch);
/* Algorithmic HBM bytes of one launch of that kernel over all problems. */
int tog_batch_kernel_bytes(tog_batch* b, int32_t kernel, double* bytes);

/* ---- learned warm start (no counterpart in TopOpt.jl) -----------------------------------
 * A 3D convolutional encoder-decoder (4 levels, 16/32/48/64 channels, 3x3x3 kernels, BF16
 * weights and activations with FP32 accumulation on the tensor cores) for a structured
 * node grid of nodes[0] x nodes[1] x nodes[2] (x fastest), trained and evaluated on the
 * GPU by the library's own kernels.  Tensors are FP32, channels-last, on the device:
 * input batch x nodes x 8 (new filtered density, its change, previous displacement /
 * max |u| (3), residual f - K(new densities) u / max |residual| (3); densities averaged
 * from the cells to the nodes),
 * output / target batch x nodes x 3 (displacement correction / scale).  Parameters are
 * one FP32 vector: per layer W[cout][27][cin] then b[cout]. */
typedef struct tog_nn tog_nn;
int tog_nn_create(const int32_t nodes[3], int32_t batch, uint64_t seed, tog_nn** out);
int tog_nn_destroy(tog_nn* nn);
int tog_nn_set_stream(tog_nn* nn, void* stream);
int tog_nn_param_count(const tog_nn* nn, int64_t* count);
int tog_nn_get_params(tog_nn* nn, float* params);
/* Also resets the optimiser state. */
int tog_nn_set_params(tog_nn* nn, const float* params);
/* Runs the network and synchronises its stream.  The convolutions run on the tcgen05 tensor
 * cores with bounded waits: a wait that gives up makes this and every later tog_nn_forward /
 * tog_nn_gradients / tog_nn_train_step (with a loss) call of the network return TOG_ERR_CUDA. */
int tog_nn_forward(tog_nn* nn, const float* in_dev, float* out_dev);
/* Mean squared error against target_dev and its gradient w.r.t. every parameter (host
 * vector of tog_nn_param_count floats; may be NULL); no update. */
int tog_nn_gradients(tog_nn* nn, const float* in_dev, const float* target_dev, double* loss, float* grads);
/* One Adam step (beta 0.9 / 0.999) on the mean squared error; loss may be NULL. */
int tog_nn_train_step(tog_nn* nn, const float* in_dev, const float* target_dev, float lr, double* loss);
/* Attach (or, with NULL, detach) a network to a 3D solver handle; it must have been created for
 * the handle's node grid with batch 1.  tog_simp_step with warm_start = TOG_WARM_LEARNED then
 * builds the network input from the handle's state on the device, runs the network and moves
 * the previous displacement u by the Galerkin step on span{d, du} (d the network's correction,
 * du the previous iteration's displacement change, r0 = f - K u), which never increases the
 * energy norm of the error; the PCG solve then finishes to the requested tolerance as before.
 * Without a previous state (first design iteration) the start is the previous displacement. */
int tog_set_warm_start_net(tog_handle* h, tog_nn* nn);
/* Keep the previous design iteration's state on the device (densities, displacement, its last
 * change) so that TOG_WARM_EXTRAPOLATE can be used without a network (3D). */
int tog_keep_previous_state(tog_handle* h);
/* Training data: the next tog_simp_step writes its network input (nodes x 8) and target (the
 * solve's displacement change / max |u_prev|, nodes x 3; the change is K^-1 of the input's
 * residual) into these FP32 device buffers, if it has a previous iteration;
 * tog_record_status reports whether it did (written = 1). */
int tog_record_next_step(tog_handle* h, float* input_dev, float* target_dev);
int tog_record_status(tog_handle* h, int32_t* written);

/* ---- allocation-free OC update: no counterpart in TopOpt.jl ----------------------------
 * For callers that cannot call cudaMalloc (a framework that owns and pre-partitions all
 * device memory, a memory-capped service, a loop that must not allocate between
 * iterations).  The update of tog_oc_update, on the caller's DEVICE arrays of n cells,
 * launched on `stream` (cudaStream_t as void*, may be NULL) without a host sync;
 * result_dev[0..2] = change, lambda, volume.  Allocates nothing: its scratch is a static
 * device array of the library (about 8.1 MiB on every GPU that loads it, held until exit),
 * so n must be <= 1,048,576 (TOG_ERR_ARG otherwise).  The first call on a device looks up
 * the array's address (make it before any stream capture) and keeps it for the process,
 * so do not call cudaDeviceReset between calls.  Calls share the array; calls that overlap
 * on the GPU race.  Having no handle, it does not hold the cells of tog_set_fixed_elements:
 * every cell is free (pass a design with fixed cells to tog_oc_update instead).  Its 100
 * bisection launches are all issued; those after convergence return at once. */
int tog_oc_update_noalloc(int64_t n, const double* x_dev, const double* dc_dev, const double* dv_dev,
                          const double* w_dev, double volfrac, double move, double* xnew_dev, double* result_dev,
                          void* stream);

#ifdef __cplusplus
}
#endif
#endif
