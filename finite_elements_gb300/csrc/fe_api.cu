// The C ABI (include/fe_gb300.h): argument checks, host<->device copies and the
// order of the assembly steps.  No arithmetic of the path runs on the host.
#include <stdio.h>
#include <string.h>

#include <algorithm>
#include <string>
#include <vector>

#include "fe_internal.h"

namespace fe {

static thread_local std::string g_last_error;

void set_error(const std::string &msg) { g_last_error = msg; }

template <typename T>
static int upload(DBuf<T> &buf, const T *host, int64_t n, cudaStream_t s) {
    FE_CHECK(dalloc(buf, (size_t)std::max<int64_t>(n, 1)));
    if (n > 0) {
        if (!host) {
            set_error("null input pointer");
            return FE_BAD_INPUT;
        }
        FE_CUDA(cudaMemcpyAsync(buf.p, host, n * sizeof(T), cudaMemcpyHostToDevice, s));
    }
    return FE_OK;
}

static void invalidate_values(fe_handle_s *h) {
    h->k_ready = h->m_ready = h->f_ready = h->sys_ready = false;
    h->have_solution = false;
    h->w.lmax[0] = h->w.lmax[1] = 0.0;
}

}  // namespace fe

using namespace fe;

#define FE_HANDLE_CHECK(h)                       \
    do {                                         \
        if (!(h)) {                              \
            set_error("null handle");            \
            return FE_BAD_INPUT;                 \
        }                                        \
    } while (0)

extern "C" {

int fe_version(void) { return 1; }

int fe_set_device(int32_t device) {
    int n = 0;
    if (cudaGetDeviceCount(&n) != cudaSuccess) {
        set_error("fe_set_device: no CUDA device");
        return FE_CUDA_ERR;
    }
    if (device < 0 || device >= n) {
        set_error("fe_set_device: device index out of range");
        return FE_BAD_INPUT;
    }
    if (cudaSetDevice(device) != cudaSuccess) {
        set_error("fe_set_device: cudaSetDevice failed");
        return FE_CUDA_ERR;
    }
    return FE_OK;
}

int fe_host_register(void *ptr, uint64_t bytes) {
    if (!ptr || bytes == 0) {
        set_error("fe_host_register: null or empty buffer");
        return FE_BAD_INPUT;
    }
    FE_CUDA(cudaHostRegister(ptr, (size_t)bytes, cudaHostRegisterDefault));
    return FE_OK;
}

int fe_host_unregister(void *ptr) {
    if (!ptr) {
        set_error("fe_host_unregister: null buffer");
        return FE_BAD_INPUT;
    }
    FE_CUDA(cudaHostUnregister(ptr));
    return FE_OK;
}

const char *fe_status_string(int status) {
    switch (status) {
        case FE_OK: return "FE_OK";
        case FE_MAXITER: return "FE_MAXITER";
        case FE_BREAKDOWN: return "FE_BREAKDOWN";
        case FE_NONFINITE: return "FE_NONFINITE";
        case FE_BAD_INPUT: return "FE_BAD_INPUT";
        case FE_CUDA_ERR: return "FE_CUDA_ERR";
        case FE_NOT_READY: return "FE_NOT_READY";
        default: return "FE_UNKNOWN";
    }
}

const char *fe_last_error(void) { return g_last_error.c_str(); }

int fe_mesh_create(int32_t kind, int64_t n_nodes, int64_t n_elem, const double *coords_host,
                   const int32_t *conn_host, fe_handle *out) {
    if (!out) {
        set_error("fe_mesh_create: null output handle");
        return FE_BAD_INPUT;
    }
    *out = nullptr;
    if (kind != FE_KIND_ELASTIC_TRI && kind != FE_KIND_MAGNETIC_TRI && kind != FE_KIND_ELASTIC_TET) {
        set_error("fe_mesh_create: unknown element kind");
        return FE_BAD_INPUT;
    }
    const int npe = kind == FE_KIND_ELASTIC_TET ? 4 : 3;
    // incidence codes element*npe + local vertex are int32
    if (n_nodes < 0 || n_elem < 0 || n_nodes > 0x3fffffffLL || n_elem * npe > 0x7fffffffLL) {
        set_error("fe_mesh_create: sizes out of range");
        return FE_BAD_INPUT;
    }
    fe_handle_s *h = new fe_handle_s();
    h->kind = kind;
    h->dim = kind == FE_KIND_ELASTIC_TRI ? 2 : kind == FE_KIND_ELASTIC_TET ? 3 : 1;
    h->npe = npe;
    h->cdim = kind == FE_KIND_ELASTIC_TET ? 3 : 2;
    h->n_nodes = n_nodes;
    h->n_elem = n_elem;
    h->n_dof = n_nodes * h->dim;
    auto fail = [&](int st) {
        fe_destroy(h);
        return st;
    };
    if (cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking) != cudaSuccess) {
        set_error("fe_mesh_create: cannot create a CUDA stream (no usable GPU?)");
        delete h;
        return FE_CUDA_ERR;
    }
    for (auto &e : h->events)
        if (cudaEventCreate(&e) != cudaSuccess) return fail(FE_CUDA_ERR);
    if (cudaMallocHost((void **)&h->err_host, sizeof(int)) != cudaSuccess) return fail(FE_CUDA_ERR);
    int st = dalloc(h->err, 1);
    if (st) return fail(st);
    if (cudaMemsetAsync(h->err.p, 0, sizeof(int), h->stream) != cudaSuccess) return fail(FE_CUDA_ERR);
    if ((st = upload(h->coords, coords_host, n_nodes * h->cdim, h->stream))) return fail(st);
    if ((st = upload(h->conn, conn_host, n_elem * npe, h->stream))) return fail(st);
    if ((st = validate_mesh(h))) return fail(st);
    *out = h;
    return FE_OK;
}

int fe_destroy(fe_handle h) {
    if (!h) return FE_OK;
    if (h->stream) cudaStreamSynchronize(h->stream);
    release_solver(h);
    dfree(h->coords), dfree(h->conn), dfree(h->E), dfree(h->nu), dfree(h->thick), dfree(h->rho), dfree(h->mu);
    dfree(h->nl_dof), dfree(h->nl_seq), dfree(h->nl_val), dfree(h->ls_ptr), dfree(h->ls_elems);
    dfree(h->ls_val), dfree(h->ls_area_total), dfree(h->ls_dim), dfree(h->ls_of_occ);
    dfree(h->bc_dof), dfree(h->bc_val), dfree(h->bc_of_dof);
    dfree(h->inc_ptr), dfree(h->inc), dfree(h->blk_ptr), dfree(h->blk_col), dfree(h->blk_row);
    dfree(h->cand), dfree(h->counts), dfree(h->scan_tmp);
    dfree(h->ke), dfree(h->me_scale), dfree(h->kval), dfree(h->mval), dfree(h->aval), dfree(h->aval32);
    dfree(h->dinv), dfree(h->dinv32), dfree(h->srow), dfree(h->sell_off), dfree(h->sell_col), dfree(h->sell_dcol), dfree(h->sell_over);
    dfree(h->sell_val64), dfree(h->sell_val32), dfree(h->diag64), dfree(h->diag32), dfree(h->dblk32), dfree(h->F), dfree(h->b), dfree(h->load_seq), dfree(h->lambda);
    dfree(h->add_dof), dfree(h->add_ptr), dfree(h->add_val), dfree(h->comp_ptr), dfree(h->comp_dof), dfree(h->comp_s);
    dfree(h->err);
    if (h->err_host) cudaFreeHost(h->err_host);
    for (auto &e : h->events)
        if (e) cudaEventDestroy(e);
    if (h->stream) cudaStreamDestroy(h->stream);
    if (h->mg_pinned) cudaFreeHost(h->mg_pinned);
    delete h;
    return FE_OK;
}

int fe_set_elastic_materials(fe_handle h, const double *E, const double *nu, const double *thickness,
                             const double *rho, int32_t plane_mode) {
    FE_HANDLE_CHECK(h);
    if (h->kind != FE_KIND_ELASTIC_TRI && h->kind != FE_KIND_ELASTIC_TET) {
        set_error("fe_set_elastic_materials: not an elasticity mesh");
        return FE_BAD_INPUT;
    }
    if (plane_mode != FE_PLANE_STRESS && plane_mode != FE_PLANE_STRAIN) {
        set_error("fe_set_elastic_materials: plane_mode must be FE_PLANE_STRESS or FE_PLANE_STRAIN");
        return FE_BAD_INPUT;
    }
    FE_CHECK(upload(h->E, E, h->n_elem, h->stream));
    FE_CHECK(upload(h->nu, nu, h->n_elem, h->stream));
    if (h->kind == FE_KIND_ELASTIC_TRI || thickness) FE_CHECK(upload(h->thick, thickness, h->n_elem, h->stream));
    h->have_rho = rho != nullptr;
    if (rho) FE_CHECK(upload(h->rho, rho, h->n_elem, h->stream));
    h->plane = plane_mode;
    h->have_material = true;
    invalidate_values(h);
    FE_CUDA(cudaStreamSynchronize(h->stream));
    return FE_OK;
}

int fe_set_mu(fe_handle h, const double *mu) {
    FE_HANDLE_CHECK(h);
    if (h->kind != FE_KIND_MAGNETIC_TRI) {
        set_error("fe_set_mu: not a magnetostatic mesh");
        return FE_BAD_INPUT;
    }
    FE_CHECK(upload(h->mu, mu, h->n_elem, h->stream));
    h->have_material = true;
    invalidate_values(h);
    FE_CUDA(cudaStreamSynchronize(h->stream));
    return FE_OK;
}

int fe_set_node_loads(fe_handle h, int64_t n, const int64_t *dof, const double *value, const int64_t *seq) {
    FE_HANDLE_CHECK(h);
    if (n < 0) {
        set_error("fe_set_node_loads: negative count");
        return FE_BAD_INPUT;
    }
    FE_CHECK(upload(h->nl_dof, dof, n, h->stream));
    FE_CHECK(upload(h->nl_val, value, n, h->stream));
    FE_CHECK(upload(h->nl_seq, seq, n, h->stream));
    h->n_node_loads = n;
    h->f_ready = h->sys_ready = false;
    FE_CUDA(cudaStreamSynchronize(h->stream));
    return FE_OK;
}

int fe_set_element_loads(fe_handle h, int64_t n_sets, const int64_t *set_ptr, const int64_t *elements,
                         const double *set_value, const int32_t *set_dim, int64_t seq_base) {
    FE_HANDLE_CHECK(h);
    if (n_sets < 0 || (n_sets > 0 && !set_ptr)) {
        set_error("fe_set_element_loads: bad set list");
        return FE_BAD_INPUT;
    }
    if (n_sets > 0 && h->kind == FE_KIND_ELASTIC_TET) {
        set_error("fe_set_element_loads: element loads need element_to_node_factors and an area, which the "
                  "reference defines for triangles only");
        return FE_BAD_INPUT;
    }
    if (n_sets == 0) {
        h->n_load_sets = h->n_load_elems = 0;
        h->load_seq_base = seq_base;
        h->f_ready = h->sys_ready = false;
        return FE_OK;
    }
    int64_t n_occ = set_ptr[n_sets];
    for (int64_t s = 0; s < n_sets; ++s)
        if (set_ptr[s + 1] < set_ptr[s] || set_ptr[0] != 0) {
            set_error("fe_set_element_loads: set pointers must start at 0 and not decrease");
            return FE_BAD_INPUT;
        }
    for (int64_t s = 0; s < n_sets; ++s)
        if (set_ptr[s + 1] == set_ptr[s]) {
            // sum() over no element is 0 and the reference divides by it
            set_error("fe_set_element_loads: an ElementsLoad without elements (zero total area)");
            return FE_BAD_INPUT;
        }
    FE_CHECK(upload(h->ls_ptr, set_ptr, n_sets + 1, h->stream));
    FE_CHECK(upload(h->ls_elems, elements, n_occ, h->stream));
    FE_CHECK(upload(h->ls_val, set_value, n_sets, h->stream));
    FE_CHECK(upload(h->ls_dim, set_dim, n_sets, h->stream));
    h->n_load_sets = n_sets;
    h->n_load_elems = n_occ;
    h->load_seq_base = seq_base;
    h->f_ready = h->sys_ready = false;
    FE_CUDA(cudaStreamSynchronize(h->stream));
    return FE_OK;
}

int fe_set_dirichlet(fe_handle h, int64_t n_bc, const int64_t *dof, const double *value) {
    FE_HANDLE_CHECK(h);
    if (n_bc < 0) {
        set_error("fe_set_dirichlet: negative count");
        return FE_BAD_INPUT;
    }
    FE_CHECK(upload(h->bc_dof, dof, n_bc, h->stream));
    FE_CHECK(upload(h->bc_val, value, n_bc, h->stream));
    h->bc_dof_host.assign(dof, dof + n_bc);
    h->n_bc = n_bc;
    h->sys_ready = false;
    h->have_solution = false;
    h->w.lmax[0] = h->w.lmax[1] = 0.0;
    FE_CUDA(cudaStreamSynchronize(h->stream));
    return FE_OK;
}

int fe_element_node_factors(fe_handle h, int64_t n, const int64_t *elements, double *factors) {
    FE_HANDLE_CHECK(h);
    if (h->kind == FE_KIND_ELASTIC_TET) {
        set_error("fe_element_node_factors: the reference defines element_to_node_factors for triangles only");
        return FE_BAD_INPUT;
    }
    if (n <= 0) return FE_OK;
    DBuf<int64_t> el;
    DBuf<double> out;
    int st = upload(el, elements, n, h->stream);
    if (!st) st = dalloc(out, (size_t)n * 3);
    if (!st) st = element_node_factors(h, n, el.p, out.p);
    if (!st && cudaMemcpyAsync(factors, out.p, n * 3 * sizeof(double), cudaMemcpyDeviceToHost, h->stream) != cudaSuccess)
        st = FE_CUDA_ERR;
    if (!st && cudaStreamSynchronize(h->stream) != cudaSuccess) st = FE_CUDA_ERR;
    dfree(el), dfree(out);
    return st;
}

int fe_assemble(fe_handle h, int32_t flags) {
    FE_HANDLE_CHECK(h);
    if ((flags & (FE_ASSEMBLE_K | FE_ASSEMBLE_M)) && !h->have_material) {
        set_error("fe_assemble: materials not set");
        return FE_NOT_READY;
    }
    FE_CUDA(cudaEventRecord(h->events[4], h->stream));
    if (flags & FE_ASSEMBLE_PATTERN) h->pattern_ready = false;
    FE_CHECK(build_pattern(h));
    if (flags & FE_ASSEMBLE_K) {
        FE_CHECK(assemble_stiffness(h));
        h->sys_ready = false;
    }
    if (flags & FE_ASSEMBLE_M) FE_CHECK(assemble_mass(h));
    if (flags & FE_ASSEMBLE_F) {
        FE_CHECK(assemble_loads(h));
        h->sys_ready = false;
    }
    if (h->k_ready && h->f_ready && !h->sys_ready) {
        h->singular = false;
        FE_CHECK(apply_dirichlet(h));
    }
    FE_CUDA(cudaEventRecord(h->events[5], h->stream));
    int err = check_error_word(h, "fe_assemble");
    if (err != FE_OK) {
        // nothing assembled from bad input may be used by a later export or solve
        h->k_ready = h->m_ready = h->f_ready = h->sys_ready = false;
        return err;
    }
    float ms = 0;
    FE_CUDA(cudaEventElapsedTime(&ms, h->events[4], h->events[5]));
    h->last_assemble_ms = ms;
    return FE_OK;
}

int fe_export_sizes(fe_handle h, int32_t which, int64_t *nrows, int64_t *ncols, int64_t *nnz) {
    FE_HANDLE_CHECK(h);
    if (!h->pattern_ready) {
        set_error("fe_export_sizes: assemble first");
        return FE_NOT_READY;
    }
    return export_sizes(h, which, nrows, ncols, nnz);
}

int fe_export_csr(fe_handle h, int32_t which, int64_t *indptr, int32_t *indices, double *data) {
    FE_HANDLE_CHECK(h);
    if (!h->pattern_ready) {
        set_error("fe_export_csr: assemble first");
        return FE_NOT_READY;
    }
    if (which == FE_MAT_K_AUGMENTED && h->n_bc > 0 && !h->sys_ready) {
        set_error("fe_export_csr: the augmented matrix needs K and F assembled with the conditions set");
        return FE_NOT_READY;
    }
    return export_csr(h, which, indptr, indices, data);
}

int fe_export_rhs(fe_handle h, double *rhs) {
    FE_HANDLE_CHECK(h);
    if (!h->f_ready) {
        set_error("fe_export_rhs: loads not assembled");
        return FE_NOT_READY;
    }
    if (h->n_dof > 0)
        FE_CUDA(cudaMemcpyAsync(rhs, h->F.p, h->n_dof * sizeof(double), cudaMemcpyDeviceToHost, h->stream));
    if (h->n_bc > 0)
        FE_CUDA(cudaMemcpyAsync(rhs + h->n_dof, h->bc_val.p, h->n_bc * sizeof(double), cudaMemcpyDeviceToHost,
                                h->stream));
    FE_CUDA(cudaStreamSynchronize(h->stream));
    return FE_OK;
}

int fe_export_element_matrices(fe_handle h, int32_t which, double *out) {
    FE_HANDLE_CHECK(h);
    return export_element_matrices(h, which, out);
}

int fe_solve(fe_handle h, const fe_solve_opts *opts, double *x_host, fe_solve_stats *stats) {
    FE_HANDLE_CHECK(h);
    fe_solve_opts def;
    memset(&def, 0, sizeof(def));
    if (!opts) opts = &def;
    fe_solve_stats local;
    memset(&local, 0, sizeof(local));
    int st = solve(h, opts, &local);
    if (stats) *stats = local;
    if (st != FE_OK) return st;
    if (x_host) FE_CHECK(fe_get_solution(h, x_host));
    return local.status;
}

int fe_get_solution(fe_handle h, double *x) {
    FE_HANDLE_CHECK(h);
    if (!h->have_solution) {
        set_error("fe_get_solution: no solution yet");
        return FE_NOT_READY;
    }
    if (h->n_dof > 0)
        FE_CUDA(cudaMemcpyAsync(x, h->w.x.p, h->n_dof * sizeof(double), cudaMemcpyDeviceToHost, h->stream));
    if (h->n_bc > 0)
        FE_CUDA(cudaMemcpyAsync(x + h->n_dof, h->lambda.p, h->n_bc * sizeof(double), cudaMemcpyDeviceToHost,
                                h->stream));
    FE_CUDA(cudaStreamSynchronize(h->stream));
    // continuity multipliers after the Dirichlet ones (rows n_dof + n_bc + k)
    for (int64_t k = 0; k < h->n_cont; ++k) x[h->n_dof + h->n_bc + k] = h->mu_host[(size_t)k];
    return FE_OK;
}

int fe_solution_device_ptr(fe_handle h, const double **ptr) {
    FE_HANDLE_CHECK(h);
    if (!h->have_solution) {
        set_error("fe_solution_device_ptr: no solution yet");
        return FE_NOT_READY;
    }
    *ptr = h->w.x.p;
    return FE_OK;
}

int fe_set_l2_keep(fe_handle h, int64_t bytes) {
    FE_HANDLE_CHECK(h);
    if (bytes < 0) {
        set_error("fe_set_l2_keep: negative size");
        return FE_BAD_INPUT;
    }
    h->l2_keep = (uint64_t)bytes;
    return FE_OK;
}

int fe_info(fe_handle h, int64_t *n_dof, int64_t *n_bc, int64_t *n_blocks) {
    FE_HANDLE_CHECK(h);
    if (n_dof) *n_dof = h->n_dof;
    if (n_bc) *n_bc = h->n_bc;
    if (n_blocks) *n_blocks = h->nnzb;
    return FE_OK;
}

int fe_event_record(fe_handle h, int32_t slot) {
    FE_HANDLE_CHECK(h);
    if (slot < 0 || slot > 3) {
        set_error("fe_event_record: slots 0..3 are free for callers");
        return FE_BAD_INPUT;
    }
    FE_CUDA(cudaEventRecord(h->events[slot], h->stream));
    return FE_OK;
}

int fe_event_elapsed_ms(fe_handle h, int32_t a, int32_t b, double *ms) {
    FE_HANDLE_CHECK(h);
    if (a < 0 || a > 3 || b < 0 || b > 3) {
        set_error("fe_event_elapsed_ms: slots 0..3");
        return FE_BAD_INPUT;
    }
    FE_CUDA(cudaEventSynchronize(h->events[b]));
    float t = 0;
    FE_CUDA(cudaEventElapsedTime(&t, h->events[a], h->events[b]));
    *ms = t;
    return FE_OK;
}

int fe_synchronize(fe_handle h) {
    FE_HANDLE_CHECK(h);
    FE_CUDA(cudaStreamSynchronize(h->stream));
    return FE_OK;
}

int fe_launch_count(fe_handle h, int64_t *count) {
    FE_HANDLE_CHECK(h);
    if (count) *count = h->launches;
    return FE_OK;
}

int fe_autotune_spmv(fe_handle h, int32_t precision, int32_t *lanes_out, double *ms_out) {
    FE_HANDLE_CHECK(h);
    int lanes = 0;
    double ms = 0;
    FE_CHECK(autotune_spmv(h, precision, &lanes, &ms));
    if (lanes_out) *lanes_out = lanes;
    if (ms_out) *ms_out = ms;
    return FE_OK;
}

int fe_time_spmv(fe_handle h, int32_t precision, int32_t lanes, int32_t reps, double *ms_out) {
    FE_HANDLE_CHECK(h);
    return time_spmv(h, precision, lanes, reps, ms_out);
}

int fe_modal(fe_handle h, int32_t which, int32_t k, double sigma, int32_t steps, int32_t precision,
             double *eigvals, double *eigvecs, double *residuals) {
    FE_HANDLE_CHECK(h);
    if (!eigvals) {
        set_error("fe_modal: null eigenvalue output");
        return FE_BAD_INPUT;
    }
    return modal(h, which, k, sigma, steps, precision, eigvals, eigvecs, residuals);
}

int fe_sell_info(fe_handle h, int64_t *n_entries, int32_t *col16) {
    FE_HANDLE_CHECK(h);
    if (!h->sys_ready) {
        set_error("fe_sell_info: assemble the system first");
        return FE_NOT_READY;
    }
    int32_t last = 0;
    if (h->n_slices > 0)
        FE_CUDA(cudaMemcpy(&last, h->sell_off.p + h->n_slices, sizeof(int32_t), cudaMemcpyDeviceToHost));
    if (n_entries) *n_entries = last;
    if (col16) *col16 = h->sell_c16 ? 1 : 0;
    return FE_OK;
}

int fe_profile_kernels(fe_handle h, int32_t enable) {
    FE_HANDLE_CHECK(h);
    return profile_kernels(h, enable);
}

int fe_profile_read(fe_handle h, int32_t precision, double *cheb_ms, int64_t *cheb_n, double *spmv_ms,
                    int64_t *spmv_n) {
    FE_HANDLE_CHECK(h);
    if (precision != FE_PREC_FP64 && precision != FE_PREC_MIXED && precision != FE_PREC_MIXED_CG64) {
        set_error("fe_profile_read: unknown precision");
        return FE_BAD_INPUT;
    }
    const int slot = precision;   // graph slots follow the precision codes
    if (cheb_ms) *cheb_ms = h->w.prof_ms[slot][0];
    if (cheb_n) *cheb_n = h->w.prof_n[slot][0];
    if (spmv_ms) *spmv_ms = h->w.prof_ms[slot][1];
    if (spmv_n) *spmv_n = h->w.prof_n[slot][1];
    return FE_OK;
}

int fe_profile_read_multigrid(fe_handle h, double *smooth_ms, int64_t *smooth_n, double *setup_ms, int64_t *setups,
                              double *cycle_ms, int64_t *cycles) {
    FE_HANDLE_CHECK(h);
    if (smooth_ms) *smooth_ms = h->w.mg_ms[0];
    if (smooth_n) *smooth_n = h->w.mg_n[0];
    if (setup_ms) *setup_ms = h->w.mg_ms[1];
    if (setups) *setups = h->w.mg_n[1];
    if (cycle_ms) *cycle_ms = h->w.mg_ms[2];
    if (cycles) *cycles = h->w.mg_n[2];
    return FE_OK;
}

int fe_profile_read_multigrid_phases(fe_handle h, double *ms, int32_t n) {
    FE_HANDLE_CHECK(h);
    if (n > 0 && !ms) {
        set_error("fe_profile_read_multigrid_phases: null output");
        return FE_BAD_INPUT;
    }
    for (int k = 0; k < n && k < FE_MG_PHASES; ++k) ms[k] = h->w.mg_phase_ms[k];
    return FE_OK;
}

}  // extern "C"
