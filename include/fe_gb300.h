/*
 * fe_gb300.h -- C ABI of the GB300 (sm_103a) assembly-and-solve path for linear
 * triangles, the drop-in for finite_elements' FiniteElementAnalysis.create_matrix /
 * create_source_matrix / solve / k_matrix_sparse / m_matrix_sparse.
 *
 * All functions return an int status (FE_OK = 0).  Pointers named "host" are plain
 * host memory owned by the caller; the library copies what it needs.  Every device
 * buffer belongs to the handle and is released by fe_destroy.  fe_last_error()
 * returns a message for the last failing call on the calling thread.
 *
 * Reference interfaces replaced (paths within the reference project):
 *   finite_elements/analysis.py:617-663   create_matrix          -> fe_assemble + fe_export_csr(FE_MAT_K_AUGMENTED)
 *   finite_elements/analysis.py:665-708   create_source_matrix   -> fe_assemble + fe_export_rhs
 *   finite_elements/analysis.py:798-830   solve (scipy spsolve)  -> fe_assemble + fe_solve
 *   finite_elements/analysis.py:345-405   k/m_matrix_sparse      -> fe_export_csr(FE_MAT_K_CSC / FE_MAT_M_CSC)
 *   finite_elements/elements.py:395-536,93-118  element matrices -> fe_assemble (element kernels), fe_export_element_matrices
 *   finite_elements/elements.py:18-53,156-191   element_to_node_factors -> fe_element_node_factors
 */
#ifndef FE_GB300_H
#define FE_GB300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* status codes */
#define FE_OK          0
#define FE_MAXITER     1   /* iteration cap reached before the tolerance            */
#define FE_BREAKDOWN   2   /* p.Ap <= 0 or a singular diagonal block: not SPD        */
#define FE_NONFINITE   3   /* NaN / Inf in inputs or iterates                        */
#define FE_BAD_INPUT   4   /* argument or index out of range                         */
#define FE_CUDA_ERR    5   /* a CUDA call failed                                     */
#define FE_NOT_READY   6   /* a required earlier step (materials, assembly) missing  */

/* element kinds (finite_elements/elements.py:333 and :56) */
#define FE_KIND_ELASTIC_TRI   1   /* ElasticityTriangularElement2D, 2 DOF per node */
#define FE_KIND_MAGNETIC_TRI  2   /* MagneticElement2D, 1 DOF per node             */
#define FE_KIND_ELASTIC_TET   3   /* ElasticityTetrahedralElement3D (elements.py:663-876),
                                     3 DOF per node, 4 nodes per element              */

/* plane mode (finite_elements/elements.py:251-273) */
#define FE_PLANE_STRESS  1
#define FE_PLANE_STRAIN  2

/* fe_assemble flags */
#define FE_ASSEMBLE_K  1
#define FE_ASSEMBLE_M  2
#define FE_ASSEMBLE_F  4
#define FE_ASSEMBLE_PATTERN 8   /* rebuild the sparsity pattern even if the mesh has one */

/* matrices for fe_export_sizes / fe_export_csr */
#define FE_MAT_K_AUGMENTED  1   /* [[K, C^T], [C, 0]] in CSR, as create_matrix returns   */
#define FE_MAT_K_CSC        2   /* K without multipliers in CSC, as k_matrix_sparse      */
#define FE_MAT_M_CSC        3   /* M without multipliers in CSC, as m_matrix_sparse      */

/* fe_solve_opts.flags */
#define FE_SOLVE_ACCEPT_STAGNATION 1   /* FP64: a true residual that restarts no longer
                                          lower (rounding floor) ends the solve with FE_OK */
#define FE_SOLVE_X0_IF_BETTER     4    /* keep x0 only if its FP64 true residual is below
                                          that of the zero start (prescribed values only);
                                          fe_solve_stats.x0_used reports the choice     */
#define FE_SOLVE_RESTART_EACH_STEP 2   /* mixed: restart the Krylov space at every refinement
                                          step (classic iterative refinement) instead of
                                          continuing along the current direction          */
#define FE_SOLVE_MULTIGRID        8    /* PCG with an FP64 recurrence preconditioned by one
                                          FP32 smoothed-aggregation V-cycle per iteration
                                          (hierarchy set up on the device at every solve;
                                          Chebyshev smoothing on node-block Jacobi, 3 steps
                                          on the finest level and 2 below, a dense
                                          coarsest solve); precision and Chebyshev
                                          options are not used, x0 and
                                          FE_SOLVE_X0_IF_BETTER are                        */

/* solver precision */
#define FE_PREC_FP64   0   /* FP64 PCG: the drop-in for spsolve                            */
#define FE_PREC_MIXED  1   /* FP32 SpMV/preconditioner inside FP64 iterative refinement;
                              an FP32 iteration that stalls above tol (FP32 floor of a
                              strongly heterogeneous problem) is finished by FP64 PCG    */
#define FE_PREC_MIXED_CG64 2 /* FP64 CG recurrence (x, r, p, q, q = A p on the FP64 copy)
                              with the block-Jacobi/Chebyshev preconditioner in FP32 on
                              the FP32 copy: all but one SpMV per iteration in FP32,
                              FP64 convergence                                         */

typedef struct fe_handle_s *fe_handle;

typedef struct fe_solve_opts {
    int32_t precision;     /* FE_PREC_FP64, FE_PREC_MIXED or FE_PREC_MIXED_CG64          */
    int32_t cheb_degree;   /* <= 1: node-block Jacobi; k >= 2: k-step Chebyshev on it (k <= 128) */
    int32_t max_iter;      /* cap on PCG iterations, all refinement steps together       */
    int32_t max_outer;     /* cap on refinement steps (mixed) or restarts (FP64)          */
    double  tol;           /* target ||b - A x||_2 / ||b||_2, FP64 true residual          */
    double  inner_tol;     /* mixed: relative residual each FP32 inner solve aims for    */
    double  cheb_ratio;    /* Chebyshev interval [lmax/ratio, lmax]; <= 0 -> default     */
    const double *x0;      /* initial guess, n_dof values, or NULL for zero               */
    int32_t x0_device;     /* 1 if x0 is a device pointer                                 */
    int32_t lanes;         /* lanes per block row in SpMV: 1,2,4,8; 0 = autotuned         */
    int32_t chunk;         /* PCG iterations per graph launch; 0 = default                */
    int32_t flags;         /* FE_SOLVE_* bits                                              */
} fe_solve_opts;

typedef struct fe_solve_stats {
    int32_t status;        /* FE_OK or a failure status                                   */
    int32_t iterations;    /* PCG iterations (inner iterations summed for mixed)          */
    int32_t outer;         /* refinement steps (mixed) or true-residual restarts (FP64)   */
    int32_t spmv;          /* sparse matrix-vector products issued                        */
    double  relres;        /* final ||b - A x|| / ||b|| recomputed in FP64                 */
    double  bnorm;         /* ||b||_2 of the eliminated system                            */
    double  solve_ms;      /* device time of the solve, CUDA events on the handle stream  */
    double  assemble_ms;   /* device time of the last fe_assemble                         */
    int32_t fp64_iterations; /* mixed: iterations of the FP64 finish (0 when FP32 met tol);
                                included in iterations                                   */
    int32_t x0_used;       /* 1 if the solve started from the given x0                    */
} fe_solve_stats;

int         fe_version(void);
/* Select the GPU that the calling thread's later calls (handle creation included) use,
 * e.g. the local rank's device when one process per GPU runs replicas.  No
 * counterpart in the reference (CPU only). */
int         fe_set_device(int32_t device);
/* Page-lock (pin) a caller's host buffer so that the library's copies from and to it run
 * at the link's speed (cudaHostRegister / cudaHostUnregister); for inputs that are
 * uploaded again and again.  No counterpart in the reference (CPU only). */
int         fe_host_register(void *ptr, uint64_t bytes);
int         fe_host_unregister(void *ptr);
const char *fe_status_string(int status);
const char *fe_last_error(void);

/* Mesh: coords_host[2*n_nodes] (x, y per node, mesh.nodes order), conn_host[3*n_elem]
 * (node indices, groups then elements) for the triangle kinds; coords_host[3*n_nodes]
 * (x, y, z) and conn_host[4*n_elem] for FE_KIND_ELASTIC_TET.  Replaces the mesh walk
 * of finite_elements/analysis.py:326-338,714-735 and core.py:89-108. */
int fe_mesh_create(int32_t kind, int64_t n_nodes, int64_t n_elem,
                   const double *coords_host, const int32_t *conn_host, fe_handle *out);
int fe_destroy(fe_handle h);

/* Per-element elastic material (elements.py:229-243,380-391): E, nu, thickness,
 * rho, each n_elem values; plane_mode FE_PLANE_STRESS or FE_PLANE_STRAIN.  For
 * tetrahedra thickness is not used (may be null) and both plane modes give the same
 * isotropic 3D D (elements.py:779-796), but one must be chosen, as in the reference
 * (elements.py:265-273). */
int fe_set_elastic_materials(fe_handle h, const double *E_host, const double *nu_host,
                             const double *thickness_host, const double *rho_host,
                             int32_t plane_mode);
/* Per-element absolute permeability mu_total (elements.py:74-78). */
int fe_set_mu(fe_handle h, const double *mu_host);

/* Loads (analysis.py:457-489).  The reference keeps, for every (node, dimension), the
 * value of the LAST load in its list (analysis.py:71-110).  Each load carries its
 * position in that list as seq; the device keeps the value with the largest seq.
 * Explicit loads (user NodeLoads, halves of EdgeLoads): dof, value, seq, n of each. */
int fe_set_node_loads(fe_handle h, int64_t n, const int64_t *dof_host,
                      const double *value_host, const int64_t *seq_host);
/* ElementsLoad sets (loads.py:24-35, analysis.py:407-429): set s covers
 * elements_host[set_ptr[s] .. set_ptr[s+1]) with total value set_value[s] in 1-based
 * dimension set_dim[s].  Element occurrence k (counted over all sets in order) gives its
 * point p the sequence number seq_base + 3k + p. */
int fe_set_element_loads(fe_handle h, int64_t n_sets, const int64_t *set_ptr_host,
                         const int64_t *elements_host, const double *set_value_host,
                         const int32_t *set_dim_host, int64_t seq_base);

/* Dirichlet conditions after the reference's de-duplication (analysis.py:241-279,
 * :509-543): multiplier i constrains DOF dof_host[i] to value_host[i]. */
int fe_set_dirichlet(fe_handle h, int64_t n_bc, const int64_t *dof_host,
                     const double *value_host);

/* Additive right-hand-side entries: F[dof_k] += value_k after the loads, in list
 * order per DOF.  These are the magnet-load contributions that create_source_matrix
 * adds with += (analysis.py:556-577, :681-708; loads.py:129-147).  The reference
 * indexes them by node index, whatever the dimension. */
int fe_set_rhs_additions(fe_handle h, int64_t n, const int64_t *dof_host, const double *value_host);

/* Continuity conditions (conditions.py:196-241, analysis.py:175-199):
 * u[dof1_k] = value_k * u[dof2_k], one multiplier each; the reference uses the node
 * index as the DOF.  The conditions must link DOFs as trees (no cycle), with a finite,
 * non-zero value, and on DOFs without a Dirichlet condition (FE_BAD_INPUT at
 * fe_solve otherwise).  fe_solve then runs a projected FP64 PCG from x = 0 with the
 * node-block Jacobi preconditioner, whatever the precision, Chebyshev degree or x0
 * asked, and the solution holds n_dof + n_bc + n continuity values: u, the Dirichlet
 * multipliers, then these multipliers. */
int fe_set_continuity(fe_handle h, int64_t n, const int64_t *dof1_host, const int64_t *dof2_host,
                      const double *value_host);

/* element_to_node_factors (elements.py:18-53,156-191) of the listed elements,
 * 3 values each, written to factors_host[3*n].  Triangles only: the reference defines
 * no such factors (nor an area) for tetrahedra, so element loads and element
 * conditions on an FE_KIND_ELASTIC_TET handle return FE_BAD_INPUT. */
int fe_element_node_factors(fe_handle h, int64_t n, const int64_t *elements_host,
                            double *factors_host);

/* Element kernels, pattern build, segmented reduction, loads and Dirichlet
 * elimination on the device (create_matrix / create_source_matrix). */
int fe_assemble(fe_handle h, int32_t flags);

int fe_export_sizes(fe_handle h, int32_t which, int64_t *nrows, int64_t *ncols, int64_t *nnz);
/* Canonical sorted CSR (or CSC) with explicit zeros kept, as scipy builds it. */
int fe_export_csr(fe_handle h, int32_t which, int64_t *indptr_host, int32_t *indices_host,
                  double *data_host);
/* create_source_matrix: n_dof load entries then n_bc prescribed values. */
int fe_export_rhs(fe_handle h, double *rhs_host);
/* Element matrices, row-major (npe*dim)^2 per element (npe = 3 nodes per triangle, 4
 * per tetrahedron): which = FE_ASSEMBLE_K or _M. */
int fe_export_element_matrices(fe_handle h, int32_t which, double *out_host);

/* Solve the eliminated system with PCG and recover the multipliers
 * lambda_i = (F - K u)[dof_i].  x_host (optional) receives n_dof + n_bc values,
 * u then lambda, as solve() returns them (analysis.py:816-830), followed by the
 * n_cont continuity multipliers when fe_set_continuity set any. */
int fe_solve(fe_handle h, const fe_solve_opts *opts, double *x_host, fe_solve_stats *stats);
/* L2 residency of the FP32 preconditioner matrix (2 DOF per node): the first `bytes`
 * of its values are loaded with L2 priority evict_last and the rest evict_first, so
 * that this prefix stays in L2 from one Chebyshev step to the next.  Default 40 MB
 * (40000000); 0 = plain loads.  No counterpart in the reference. */
int fe_set_l2_keep(fe_handle h, int64_t bytes);
/* Copy the last solution (n_dof + n_bc [+ n_cont] values) to the host. */
int fe_get_solution(fe_handle h, double *x_host);
/* Device address of the last solution u (n_dof doubles), valid until the next solve. */
int fe_solution_device_ptr(fe_handle h, const double **ptr);

/* Sizes of the handle: n_dof, number of Dirichlet conditions, stored 2x2 (or 1x1)
 * blocks of K. */
int fe_info(fe_handle h, int64_t *n_dof, int64_t *n_bc, int64_t *n_blocks);

/* CUDA events on the handle's stream, for timing around library calls. */
int fe_event_record(fe_handle h, int32_t slot);
int fe_event_elapsed_ms(fe_handle h, int32_t slot_a, int32_t slot_b, double *ms);
int fe_synchronize(fe_handle h);
/* Number of this library's kernels the handle has launched so far (graph-captured
 * launches included, counted per kernel node executed). */
int fe_launch_count(fe_handle h, int64_t *count);
/* Lanes per block row the autotuner chose for SpMV in the given precision. */
int fe_autotune_spmv(fe_handle h, int32_t precision, int32_t *lanes_out, double *ms_out);
/* Average device time of one SpMV with the given lanes (reps repetitions). */
int fe_time_spmv(fe_handle h, int32_t precision, int32_t lanes, int32_t reps, double *ms_out);
/* Layout of the solver's SELL-32 copies (no counterpart in the reference): stored
 * entries (padding included) and whether the FP32 kernels read 16-bit column offsets
 * (1) or the int32 columns (0, some offset exceeds 32767). */
int fe_sell_info(fe_handle h, int64_t *n_entries, int32_t *col16);
/* Kernel timing inside the solver's captured PCG loop (no counterpart in the
 * reference; for measurement).  enable = 1 adds CUDA event records to the first
 * iteration of every 16-iteration chunk -- around the run of intermediate Chebyshev
 * steps 2 .. k-2 (degree >= 4) and around the PCG SpMV -- and resets the sums; 0
 * removes them.  fe_profile_read returns, for the given precision, the summed device
 * time (ms) and the number of launches it covers, for the Chebyshev steps and for the
 * PCG SpMV. */
int fe_profile_kernels(fe_handle h, int32_t enable);
int fe_profile_read(fe_handle h, int32_t precision, double *cheb_ms, int64_t *cheb_n, double *spmv_ms,
                    int64_t *spmv_n);
/* The multigrid solve's times summed since fe_profile_kernels(h, 1): level 0's
 * pre-smoothing in the V-cycle (ms, and its Chebyshev launches), the device setup of the
 * hierarchy (ms, solves) and the whole V-cycle (ms, cycles); events recorded inside the
 * captured cycle and read after each of its launches. */
int fe_profile_read_multigrid(fe_handle h, double *smooth_ms, int64_t *smooth_n, double *setup_ms, int64_t *setups,
                              double *cycle_ms, int64_t *cycles);
/* The multigrid setup's time per phase (ms, summed over levels and solves since
 * fe_profile_kernels(h, 1)), into ms[0 .. min(n, FE_MG_PHASES)):
 *   0 level 0's copy of the operator and near-null space, 1 D^-1 and the power
 *   iterations, 2 aggregation (strength, distance-2 independent set, joins), 3 member
 *   lists and per-aggregate QR, 4 A P_t and the smoothing of P, 5 A P, 6 P^T, 7 the
 *   Galerkin product P^T (A P), 8 the coarsest dense inverse, 9 the cycle's FP32 copies
 *   and graph capture.
 * Stream time between events recorded where each phase starts (host work and waits
 * included). */
#define FE_MG_PHASES 10
int fe_profile_read_multigrid_phases(fe_handle h, double *ms, int32_t n);
/* The multigrid solve allocates from one stream-ordered memory pool per device, shared
 * by the process's handles, which keeps its memory between solves and handles (no page
 * mapping and no device-wide synchronisation per allocation).  This gives the pools'
 * unused memory back to the device down to keep_bytes each (cudaMemPoolTrimTo). */
int fe_trim_memory_pools(uint64_t keep_bytes);

/* ---- modal analysis (analysis.py:741-796 modal_analysis: scipy eigsh/eigs on
 * k_matrix_sparse and m_matrix_sparse, i.e. K and M without Dirichlet conditions).
 * Needs K and M assembled (FE_ASSEMBLE_K | FE_ASSEMBLE_M).  Shift-invert Lanczos in
 * the M inner product (which = FE_MODAL_SMALLEST: the k smallest eigenvalues of
 * K v = lambda M v, rigid-body zeros included; sigma < 0 is the shift, 0 or NaN picks
 * one) or Lanczos on M^-1 K (FE_MODAL_LARGEST).  Each step solves with the library's
 * PCG (precision FE_PREC_FP64 or FE_PREC_MIXED_CG64).  steps: Lanczos steps (0 =
 * default).  Output, by increasing eigenvalue: eigvals_host[k]; eigvecs_host[k][n_dof]
 * (unit 2-norm) or NULL; residuals_host[k] = ||K x - lambda M x|| /
 * (||K x|| + max(|lambda|, |lambda|max) ||M x||) or NULL, |lambda|max the largest of
 * the k.  The static system (K with the conditions) is rebuilt by the next fe_solve. */
#define FE_MODAL_SMALLEST 0
#define FE_MODAL_LARGEST  1
int fe_modal(fe_handle h, int32_t which, int32_t k, double sigma, int32_t steps, int32_t precision,
             double *eigvals_host, double *eigvecs_host, double *residuals_host);

/* ---- post-processing of a solution (results.py:809-830 strain/stress, :769-781 and
 * elements.py:275-292 energy, results.py:121-152 magnetic field).  u_host / a_host:
 * n_dof values, or NULL for the handle's last solution.  Per element: strain and
 * stress 3 values each (xx, yy, xy), energy 1; magnetic field 2 (Bx, By).  On a
 * tetrahedral handle strain and stress have 6 values each (xx, yy, zz, xy, yz, zx:
 * the rows of the 3D B, elements.py:719-748). */
int fe_post_elastic(fe_handle h, const double *u_host, double *strain_host, double *stress_host,
                    double *energy_host);
int fe_post_magnetic(fe_handle h, const double *a_host, double *field_host);

/* ---- smoothed-aggregation multigrid setup on the host (no counterpart in the
 * reference, which factorises directly; the setup stage of a multilevel preconditioner
 * for the device solve).  Input: the node-block CSR of a symmetric system matrix
 * (n_nodes block rows of d x d blocks, blk_ptr[n_nodes+1], blk_col, vals row-major
 * blocks) and a near-null space (n_nodes*d x m, row-major: the rigid-body modes for
 * elasticity).  Levels down to at most coarse_dofs DOFs (or 12).  Level l < n_levels
 * has its matrix (which = 0, d_l x d_l blocks) and its prolongator (which = 1, d_l x m
 * blocks, columns = aggregates); level n_levels is the coarsest matrix. */
typedef struct fe_amg_s *fe_amg;
int fe_amg_build_host(int64_t n_nodes, int32_t d, const int64_t *blk_ptr, const int32_t *blk_col,
                      const double *vals, int32_t m, const double *nullspace, double theta,
                      int64_t coarse_dofs, fe_amg *out);
/* The same, set up by the passes of the device setup run on the host: aggregates from a
 * distance-2 maximal independent set of the strong graph (rounds of (state, hash,
 * index) maxima over two hops; every node then joins the strongest root next to it, the
 * rest the strongest neighbour that joined), one QR per aggregate, row-wise sparse
 * products (sorted distinct columns, then the values).  Its result does not depend on
 * the order in which rows are processed. */
int fe_amg_build_parallel_host(int64_t n_nodes, int32_t d, const int64_t *blk_ptr, const int32_t *blk_col,
                               const double *vals, int32_t m, const double *nullspace, double theta,
                               int64_t coarse_dofs, fe_amg *out);
/* The same passes on the device, from the assembled system of h (near-null space: the
 * rigid-body modes, or the constant for magnetostatics, zero on the constrained DOFs),
 * with the coarsest inverse computed on the device; the hierarchy is copied to the host
 * for the accessors below. */
int fe_amg_build_device(fe_handle h, double theta, int64_t coarse_dofs, fe_amg *out);
int fe_amg_levels(fe_amg a, int32_t *n_levels);
int fe_amg_level_info(fe_amg a, int32_t level, int64_t *n_nodes, int32_t *d, int64_t *nnzb_A,
                      int64_t *nnzb_P, int64_t *n_coarse, int32_t *m, double *lmax);
int fe_amg_level_matrix(fe_amg a, int32_t level, int32_t which, int64_t *ptr_host, int32_t *col_host,
                        double *val_host);
int fe_amg_level_aggregates(fe_amg a, int32_t level, int32_t *agg_host);
/* One V-cycle x = M^-1 r on the host with k_smooth Chebyshev steps (on D^-1 A over
 * [1.05 lmax/30, 1.05 lmax]) before and after each coarse correction and a dense solve
 * of the coarsest level: the arithmetic the device cycle runs row by row. */
int fe_amg_vcycle_host(fe_amg a, int32_t k_smooth, const double *r_host, double *x_host);
/* The device's FP32 cycle (FP32 copies of the levels, r rounded to FP32, FP64 coarsest
 * inverse) run on the host: the sequence of passes the multigrid solve launches. */
int fe_amg_vcycle_host_f32(fe_amg a, int32_t k_smooth, const double *r_host, double *x_host);
/* The device's multigrid PCG (FP64 recurrence around the FP32 cycle) run on the host on
 * the hierarchy's level-0 matrix: x (host, n DOFs) from zero to ||r|| <= tol ||b||;
 * iterations, the true relative residual and the status (FE_OK, FE_MAXITER,
 * FE_BREAKDOWN, FE_NONFINITE) come back through the pointers. */
int fe_amg_pcg_host(fe_amg a, int32_t k_smooth, const double *b_host, double tol, int32_t max_iter, double *x_host,
                    int32_t *iterations, double *relres, int32_t *status);
int fe_amg_destroy(fe_amg a);

/* ---- learned warm start (no counterpart in the reference: an addition on top of the
 * PCG that replaces spsolve in analysis.py:816-830; PCG from its x0 still decides
 * the accuracy).  A graph network over the mesh nodes (6 message-passing layers,
 * hidden width 64, BF16 tensor-core GEMMs with FP32 accumulation) predicts the shape
 * u_hat of the displacement; x0 = g + s u_hat with s the A-norm optimal scale.
 * Elasticity meshes only. */
typedef struct fe_gnn_s *fe_gnn;
int fe_gnn_create(fe_gnn *out);
int fe_gnn_destroy(fe_gnn g);
int fe_gnn_num_params(int64_t *n);
int fe_gnn_set_params(fe_gnn g, const float *params_host, int64_t n);
int fe_gnn_get_params(fe_gnn g, float *params_host, int64_t n);
/* The 16 node features of an assembled handle, n_nodes x 16 FP32. */
int fe_gnn_features(fe_gnn g, fe_handle h, float *features_host);  /* see fe_gnn.cu k_features */
/* Warm start for h: *x0_dev (device, n_dof doubles, owned by g, valid until the next
 * call; a copy also goes to x0_host when not NULL) and the scale s.  Pass *x0_dev to
 * fe_solve as opts.x0 with opts.x0_device = 1. */
int fe_gnn_predict(fe_gnn g, fe_handle h, double *x0_host, const double **x0_dev, double *scale);
/* The same prediction enqueued on the network's own stream without waiting for it: it
 * starts after the handle's work so far (the assembly) and the handle's next solve waits
 * for it just before it reads opts.x0, so a solve's multigrid setup overlaps with it.
 * *x0_dev (n_dof doubles) is valid for that solve; the scale stays on the device.  Call
 * a solve of h (or fe_synchronize on it) before the next prediction or destroying g. */
int fe_gnn_predict_async(fe_gnn g, fe_handle h, const double **x0_dev);
/* Training target of h's last solution: b~ . (x - g), the energy of its free part. */
int fe_gnn_target_energy(fe_gnn g, fe_handle h, double *energy);
/* Loss 1 - (u.b~)^2 / ((u.A u) energy) and its gradient w.r.t. every parameter
 * (kept on the device for fe_gnn_adam_step; copied to grad_host when not NULL). */
int fe_gnn_loss_grad(fe_gnn g, fe_handle h, double energy, double *loss, float *grad_host);
/* Mean-squared error of u_hat against h's last solution, (x - g) / RMS(x - g) on the
 * free DOFs, and its gradient (the training loss; gradient kept as above). */
int fe_gnn_fit_grad(fe_gnn g, fe_handle h, double *loss, float *grad_host);
int fe_gnn_adam_step(fe_gnn g, float lr, float beta1, float beta2, float eps);

/* ---- batched solve of many independent elasticity instances (no counterpart in the
 * reference, which solves one analysis per spsolve call, analysis.py:816-830).  The
 * instances are concatenated into one handle (fe_mesh_create on the union mesh with
 * disjoint node ranges, then the usual setters and fe_assemble); node_ptr_host[i] ..
 * node_ptr_host[i+1] are instance i's nodes.  The batched solve is the mixed-precision
 * PCG of FE_PREC_MIXED_CG64 per instance -- FP64 recurrence, node-block Jacobi +
 * Chebyshev preconditioner in FP32 with each instance's own Chebyshev interval -- run by
 * one persistent cooperative kernel per chunk of iterations (grid barriers between its
 * phases, with bounded waits), replayed from a CUDA graph.  Reductions are per
 * instance and deterministic; converged instances drop out. */
typedef struct fe_batch_s *fe_batch;
int fe_batch_create(fe_handle h, int32_t n_instances, const int64_t *node_ptr_host, fe_batch *out);
int fe_batch_destroy(fe_batch b);
/* Resident blocks per SM of the persistent kernel (0 = as many as fit) and SELL slices
 * (32 node rows each) per work item of a warp. */
int fe_batch_set_tiles(fe_batch b, int32_t blocks_per_sm, int64_t slices_per_item);
/* Chebyshev terms of the preconditioner (1 = node-block Jacobi alone, up to 128) and the
 * ratio lmax / lmin of each instance's interval; default 16 and 1e4. */
int fe_batch_set_preconditioner(fe_batch b, int32_t cheb_degree, double cheb_ratio);
/* Time a chunk of iterations for each (blocks per SM, slices per item) candidate and keep
 * the fastest. */
int fe_batch_autotune(fe_batch b, int32_t *blocks_per_sm_out, int64_t *slices_per_item_out,
                      double *us_per_iter_out);
/* Solve every instance to ||b_i - A_i x_i|| <= tol ||b_i|| (FP64 true residual);
 * per-instance iterations, status and final true relative residual (each optional), the
 * union solution (n_dof values, optional) and the device time of the solve (including
 * the per-instance Chebyshev-interval probe after a new assembly). */
int fe_batch_solve(fe_batch b, double tol, int32_t max_iter, int32_t *iterations_host, int32_t *status_host,
                   double *relres_host, double *x_host, double *ms_out);
/* The last fe_batch_solve: replays of the captured chunk, launches of the persistent
 * kernel, whether chunks replay from a CUDA graph (1) or launch directly (0), and the
 * cooperative grid (each optional). */
int fe_batch_last_run(fe_batch b, int32_t *graph_launches, int32_t *kernel_launches, int32_t *uses_graph,
                      int32_t *grid);

/* No counterpart in the reference.  Exclusive scan of n int32 counts into n+1 int32
 * offsets (offsets_dev[0] = 0, offsets_dev[n] = total; -1 there if the total does not
 * fit in int32) that allocates nothing: for callers who may not call cudaMalloc --
 * those whose device memory all comes from another owner's pool, or who are on a hot
 * path where cudaMalloc/cudaFree would synchronise the device.  counts_dev and
 * offsets_dev are the caller's device buffers; stream is a cudaStream_t (NULL = the
 * default stream); the call only enqueues work.  The per-tile sums live in one fixed
 * array inside the library (256 KiB per GPU, kept until exit), so n is limited to
 * 67,108,864 (FE_BAD_INPUT beyond).  Calls that overlap on the GPU share that array
 * and race.  The first call on each device looks the array up: make it before any
 * stream capture.  That address is kept for the life of the process: after a
 * cudaDeviceReset (or any teardown of the device's primary context) this entry point
 * must not be called again in the same process.  Check offsets_dev[n] before using any
 * offset: when it is -1 the running sums passed 2^31 - 1 and the offsets after that
 * point have wrapped.  Same results as the scan behind fe_export_csr's row pointers. */
int fe_scan_counts_noalloc(const int32_t *counts_dev, int32_t *offsets_dev, int64_t n, void *stream);

#ifdef __cplusplus
}
#endif

#endif /* FE_GB300_H */
