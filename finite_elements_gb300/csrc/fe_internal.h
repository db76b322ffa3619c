// Internal state of one assembly-and-solve handle and the helpers shared by the
// translation units of libfe_gb300.so.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <string>
#include <vector>
#include <type_traits>

#include "../../include/fe_gb300.h"

namespace fe {

// ---------------------------------------------------------------- error plumbing

void set_error(const std::string &msg);

#define FE_CUDA(...)                                                                   \
    do {                                                                               \
        cudaError_t _e = (__VA_ARGS__);                                                \
        if (_e != cudaSuccess) {                                                       \
            ::fe::set_error(std::string(#__VA_ARGS__) + ": " + cudaGetErrorString(_e)); \
            return FE_CUDA_ERR;                                                        \
        }                                                                              \
    } while (0)

#define FE_CHECK(...)                                \
    do {                                             \
        int _s = (__VA_ARGS__);                      \
        if (_s != FE_OK) return _s;                  \
    } while (0)

#define FE_LAUNCH_CHECK() FE_CUDA(cudaGetLastError())

// device error word bits (set by kernels, read by the host after a step)
enum : int {
    ERR_CONN_RANGE = 1,      // connectivity index outside [0, n_nodes)
    ERR_DOF_RANGE = 2,       // load / condition DOF outside [0, n_dof)
    ERR_ELEM_RANGE = 4,      // element index outside [0, n_elem)
    ERR_NONFINITE = 8,       // NaN / Inf met
    ERR_SINGULAR_BLOCK = 16, // zero determinant in a diagonal block
    ERR_PATTERN = 32,        // a block expected in the pattern was not found
};

constexpr int kThreads = 256;

inline int grid_for(int64_t n, int threads = kThreads, int cap = 152 * 16) {
    int64_t g = (n + threads - 1) / threads;
    if (g < 1) g = 1;
    if (g > cap) g = cap;
    return (int)g;
}

// Calls f(std::integral_constant<int, D>{}) for the DOF count per node d (1, 2 or 3)
// and returns its status: one place turns the runtime d into a template argument.
template <typename F>
int with_dim(int d, F f) {
    switch (d) {
    case 1: return f(std::integral_constant<int, 1>{});
    case 2: return f(std::integral_constant<int, 2>{});
    case 3: return f(std::integral_constant<int, 3>{});
    default: return FE_BAD_INPUT;
    }
}

// ---------------------------------------------------------------- buffers

template <typename T>
struct DBuf {
    T *p = nullptr;
    size_t n = 0;
};

template <typename T>
int dalloc(DBuf<T> &b, size_t n) {
    if (b.p && b.n >= n) return FE_OK;
    if (b.p) {
        cudaFree(b.p);
        b.p = nullptr;
        b.n = 0;
    }
    if (n == 0) return FE_OK;
    FE_CUDA(cudaMalloc((void **)&b.p, n * sizeof(T)));
    b.n = n;
    return FE_OK;
}

template <typename T>
void dfree(DBuf<T> &b) {
    if (b.p) cudaFree(b.p);
    b.p = nullptr;
    b.n = 0;
}

// PCG scalars live in device memory so that every decision of the iteration is
// taken on the device (no host round trip per iteration).
struct PcgScalars {
    double rz;        // r.z of the current iterate
    double pq;        // p.Ap
    double rr;        // r.r
    double bb;        // b.b (of the system the loop solves)
    double alpha, beta;
    double tol2;      // stop when rr <= tol2 * bb
    double cheb_theta, cheb_delta;   // Chebyshev interval centre / half-width
    int iter;         // iterations done in this loop
    int max_iter;
    int done;         // 1: converged or stopped, remaining launches return at once
    int status;       // FE_OK / FE_MAXITER / FE_BREAKDOWN / FE_NONFINITE
    unsigned int ticket[8];          // last-block counters, one per reducing kernel
    double hist_alpha[64], hist_beta[64];   // first iterations, for the Lanczos estimate
};

struct SolverWork {
    // FP64 vectors (n_dof each): solution, residual, preconditioned residual,
    // direction, A p, a second z for the Chebyshev ping-pong (also scratch)
    DBuf<double> x, r, z, p, q, t;
    // FP32 vectors of the mixed inner solve (the solution stays in x, FP64); rh32 is
    // D^-1 r, the right-hand side of the prescaled FP32 Chebyshev steps
    DBuf<float> r32, z32, p32, q32, zc32, rh32;
    DBuf<double> partials;   // per-block partial sums of the reductions
    DBuf<PcgScalars> sc;
    PcgScalars *sc_host = nullptr;       // pinned mirror
    double lmax[2] = {0.0, 0.0};         // largest eigenvalue of D^-1 A, [FP64, FP32]
    int lanes[2] = {0, 0};               // autotuned SpMV lanes, [FP64, FP32]
    // captured chunk, [FP64, FP32, FP64 recurrence + FP32 preconditioner]
    cudaGraphExec_t graph[3] = {nullptr, nullptr, nullptr};
    // what each captured graph was built for
    struct Key {
        int k = -1, G = -1, chunk = -1;
        const void *x = nullptr;
        double theta = 0, delta = 0;
        bool prof = false;
        uint64_t keep = 0;
    } key[3];
    // Kernel timing inside the captured loop (fe_profile_kernels): event records in
    // the first iteration of every chunk, [slot][0] around the run of intermediate
    // Chebyshev steps 2 .. k-2, [slot][1] around the PCG SpMV (slots as graph[]);
    // summed durations and the launches they cover.
    bool prof = false;
    cudaEvent_t pev[4] = {nullptr, nullptr, nullptr, nullptr};
    double prof_ms[3][2] = {{0.0, 0.0}, {0.0, 0.0}, {0.0, 0.0}};
    // The multigrid solve's times while profiling: [0] level 0's pre-smoothing (ms, its
    // Chebyshev launches), [1] the device setup of the hierarchy (ms, solves), [2] the
    // whole V-cycle (ms, cycles)
    double mg_ms[3] = {0.0, 0.0, 0.0};
    int64_t mg_n[3] = {0, 0, 0};
    double mg_phase_ms[16] = {};   // multigrid setup time per phase (amg::SetupPhase)
    int64_t prof_n[3][2] = {{0, 0}, {0, 0}, {0, 0}};
};

}  // namespace fe

struct fe_handle_s {
    int kind = 0;            // FE_KIND_*
    int dim = 0;             // DOF per node
    int npe = 3;             // nodes per element: 3 (triangles) or 4 (tetrahedra)
    int cdim = 2;            // coordinates per node: 2 or 3
    int64_t n_nodes = 0, n_elem = 0, n_dof = 0;
    int32_t max_node = -1;   // largest node index used by an element
    cudaStream_t stream = nullptr;
    // events 0..3 belong to callers (fe_event_record); the library times its own
    // steps with 4..5 (assembly), 6..7 (solve) and 8..9 (SpMV timing)
    cudaEvent_t events[10] = {};

    // inputs
    fe::DBuf<double> coords;      // [n_nodes][cdim]
    fe::DBuf<int32_t> conn;       // [n_elem][npe]
    fe::DBuf<double> E, nu, thick, rho, mu;
    int plane = 0;
    bool have_material = false, have_rho = false;

    // loads
    int64_t n_node_loads = 0;
    fe::DBuf<int64_t> nl_dof, nl_seq;
    fe::DBuf<double> nl_val;
    int64_t n_load_sets = 0, n_load_elems = 0, load_seq_base = 0;
    fe::DBuf<int64_t> ls_ptr, ls_elems;
    fe::DBuf<double> ls_val, ls_area_total;
    fe::DBuf<int32_t> ls_dim, ls_of_occ;

    // Dirichlet conditions
    int64_t n_bc = 0;
    fe::DBuf<int64_t> bc_dof;
    fe::DBuf<double> bc_val;
    fe::DBuf<int32_t> bc_of_dof;  // [n_dof] multiplier index or -1
    std::vector<int64_t> bc_dof_host;

    // additive right-hand-side entries (magnet loads): unique DOFs, and per DOF the
    // values in list order, add_ptr[k] .. add_ptr[k+1]
    int64_t n_add_dofs = 0;
    fe::DBuf<int64_t> add_dof, add_ptr;
    fe::DBuf<double> add_val;

    // continuity conditions u[dof1] = value * u[dof2], grouped into trees of linked
    // DOFs: on a tree the admissible vectors are t * s (s_root = 1); comp_* on the
    // device for the projection, the host keeps each tree in BFS order for the
    // multipliers
    int64_t n_cont = 0, n_comp = 0;
    std::vector<int64_t> cont_d1, cont_d2;
    std::vector<double> cont_v;
    std::vector<int64_t> comp_ptr_h, comp_dof_h, comp_edge_h;   // edge to the BFS parent (-1 at roots)
    std::vector<double> comp_s_h;
    fe::DBuf<int64_t> comp_ptr, comp_dof;
    fe::DBuf<double> comp_s;
    std::vector<double> mu_host;   // continuity multipliers of the last solve

    // bytes of the FP32 SELL values kept L2-resident across Chebyshev steps (0 = off);
    // 40 MB measured best at 4M DOF (1.813 s against 1.893 s with plain loads; 80, 110,
    // 140 and 200 MB gave 1.87 s: the gathered vectors need the rest of the L2)
    uint64_t l2_keep = 40000000;

    // pattern: node-block CSR
    bool pattern_ready = false;
    fe::DBuf<int32_t> inc_ptr, inc;       // node -> (element*npe + local) incidence, sorted
    int64_t nnzb = 0;
    fe::DBuf<int32_t> blk_ptr, blk_col, blk_row;
    fe::DBuf<int32_t> cand;               // scratch for the pattern build
    fe::DBuf<int32_t> counts;             // scratch counts
    fe::DBuf<int64_t> scan_tmp;

    // values
    bool k_ready = false, m_ready = false, f_ready = false, sys_ready = false;
    uint64_t sys_generation = 0;   // counts the system matrices built (build_system)
    // memory pool of the multigrid solve's stream-ordered allocations: the device's pool,
    // shared by the process's handles and kept between solves
    cudaMemPool_t mg_pool = nullptr;
    double *mg_pinned = nullptr;   // 8 pinned doubles: the multigrid's scalar reads to the host
    // recorded by an asynchronous warm-start prediction on another stream: the next solve
    // waits for it on the handle's stream before it reads opts.x0 (start_point)
    cudaEvent_t x0_ready = nullptr;
    bool singular = false;                // a diagonal block could not be inverted
    fe::DBuf<double> ke;                  // [n_elem][(3d)^2]
    fe::DBuf<double> me_scale;            // [n_elem] rho*A*t/12
    fe::DBuf<double> kval, mval;          // [nnzb][d][d] full K / M
    fe::DBuf<double> aval;                // eliminated K (FP64)
    fe::DBuf<float> aval32;               // eliminated K (FP32, difference form)
    fe::DBuf<double> dinv;                // [n_nodes][d][d] inverse diagonal blocks
    fe::DBuf<double> srow;                // [n_nodes][d][d] block row sums of A (difference form)
    fe::DBuf<float> dinv32;
    // sliced ELL (SELL-32) copy of A for the PCG SpMVs: slice s holds 32 consecutive
    // block rows; entry k of row 32 s + l sits at sell_off[s] + 32 k + l (coalesced
    // per warp).  Off-diagonal blocks only; padding entries point at the row itself
    // with a zero block.  The diagonal lives in diag64 (A_rr) / diag32 (D^-1 S_r).
    int64_t n_slices = 0;
    fe::DBuf<int32_t> sell_off, sell_col;
    fe::DBuf<int16_t> sell_dcol;          // column offsets c - r, for the FP32 kernels
    fe::DBuf<int> sell_over;              // set when an offset does not fit in 16 bits
    bool sell_c16 = false;                // sell_dcol holds every column
    fe::DBuf<double> sell_val64, diag64;
    fe::DBuf<float> sell_val32, diag32;   // prescaled by the block-Jacobi inverse (D^-1 A_rm, D^-1 S_r)
    fe::DBuf<float> dblk32;               // [n_nodes][d][d] A_rr in FP32 (scales D^-1 A x back to A x)
    fe::DBuf<double> F;                   // loads [n_dof]
    fe::DBuf<double> b;                   // eliminated right-hand side [n_dof]
    fe::DBuf<long long> load_seq;         // [n_dof] winning load sequence
    fe::DBuf<double> lambda;              // [n_bc]
    fe::DBuf<int> err;                    // device error word
    int *err_host = nullptr;              // pinned
    double last_assemble_ms = 0.0;
    int64_t launches = 0;                 // kernels launched (graph nodes included)
    bool have_solution = false;

    fe::SolverWork w;
};

namespace fe {

// assembly (fe_assembly.cu)
int build_pattern(fe_handle_s *h);
int assemble_stiffness(fe_handle_s *h);
int assemble_mass(fe_handle_s *h);
int assemble_loads(fe_handle_s *h);
int apply_dirichlet(fe_handle_s *h);
int build_system(fe_handle_s *h, double ka, double mb, bool use_bc);
int element_node_factors(fe_handle_s *h, int64_t n, const int64_t *elems_dev, double *out_dev);
int export_sizes(fe_handle_s *h, int which, int64_t *nrows, int64_t *ncols, int64_t *nnz);
int export_csr(fe_handle_s *h, int which, int64_t *indptr, int32_t *indices, double *data);
int export_element_matrices(fe_handle_s *h, int which, double *out_host);
int check_error_word(fe_handle_s *h, const char *where);
int validate_mesh(fe_handle_s *h);
int build_sell(fe_handle_s *h);

// scan (fe_scan.cu): exclusive scan of n int32 counts into int32 offsets (n+1 values)
int exclusive_scan_i32(const int32_t *in, int32_t *out, int64_t n, int64_t *total,
                       DBuf<int64_t> &tmp, cudaStream_t s);

// solver (fe_solver.cu)
int solve(fe_handle_s *h, const fe_solve_opts *opts, fe_solve_stats *stats);
// modal analysis (fe_modal.cu)
int modal(fe_handle_s *h, int which, int k, double sigma, int steps, int precision, double *eigvals,
          double *eigvecs, double *resid);
int recover_multipliers(fe_handle_s *h);
// Continuity conditions (fe_continuity.cu): host set-up and the projected FP64 PCG
int set_continuity(fe_handle_s *h, int64_t n, const int64_t *dof1, const int64_t *dof2, const double *value);
int solve_continuity(fe_handle_s *h, const fe_solve_opts *opts, fe_solve_stats *stats);
// Largest eigenvalue of the m x m tridiagonal Lanczos matrix of the CG coefficients
// alpha[0..m), beta[0..m) (bisection on the Sturm sequence), fe_solver.cu.
double lanczos_lmax(const double *alpha, const double *beta, int m);
// The start of a solve: opts.x0 (or 0) with the prescribed values; with
// FE_SOLVE_X0_IF_BETTER the start of smaller FP64 residual (fe_solver.cu).
int solve_start_point(fe_handle_s *h, const fe_solve_opts *o, double *x, int *x0_used);
// FP64 PCG with a smoothed-aggregation V-cycle preconditioner (fe_amg_device.cu)
int solve_multigrid(fe_handle_s *h, const fe_solve_opts *opts, fe_solve_stats *stats);
int set_rhs_additions(fe_handle_s *h, int64_t n, const int64_t *dof, const double *value);
int apply_rhs_additions(fe_handle_s *h);
int autotune_spmv(fe_handle_s *h, int precision, int *lanes, double *ms);
int time_spmv(fe_handle_s *h, int precision, int lanes, int reps, double *ms);
int profile_kernels(fe_handle_s *h, int enable);
void release_solver(fe_handle_s *h);
int spmv64(fe_handle_s *h, const double *x, double *y);
// the same, enqueued on another stream (the warm-start network's)
int spmv64_on(fe_handle_s *h, const double *x, double *y, cudaStream_t stream);
// Level 0 of the multigrid V-cycle on the handle's prescaled FP32 SELL copy
// (fe_solver.cu), enqueued on the handle's stream: rh = D^-1 (float)r and
// z1 = rh * inv_theta; one Chebyshev step z_out = z_in + c1 (z_in - z_out) +
// c2 (rh - D^-1 A z_in) (first: the old iterate taken as 0); t = r - A x from rh.
int mg_level0_start(fe_handle_s *h, const double *r, float *rh, float *z1, double inv_theta);
int mg_level0_cheb(fe_handle_s *h, bool first, const float *rh, const float *zin, float *zout, double c1, double c2);
int mg_level0_residual(fe_handle_s *h, const float *rh, const float *x, float *t);

}  // namespace fe
