// The smoothed-aggregation hierarchy in device memory: set up by fe_amg_device_setup.cu,
// applied as a V-cycle by fe_amg_device.cu.
#pragma once

#include <utility>
#include <vector>

#include "fe_amg.h"
#include "fe_amg_passes.cuh"
#include "fe_internal.h"

namespace fe {

using DevCsr = amg::Csr;

// The multigrid solve's device buffers: stream-ordered allocations on the handle's
// stream from the device's memory pool, which keeps the memory between solves and
// handles, so a setup's hundred-odd allocations and frees map no pages and never
// synchronise the device.  palloc grows a buffer like dalloc; pfree returns it on the
// stream.
struct MgMem {
    cudaStream_t s = nullptr;
    cudaMemPool_t pool = nullptr;
    double *pinned = nullptr;   // 8 pinned host doubles for scalar reads (a copy to
                                // pageable memory would be staged and wait longer)
};

// the handle's stream and the device's pool (one per device for the process, created on
// first use, release threshold unbounded; fe_trim_memory_pools gives memory back)
int mg_memory(fe_handle_s *h, MgMem *out);

template <typename T>
int palloc(const MgMem &m, DBuf<T> &b, size_t n) {
    if (b.p && b.n >= n) return FE_OK;
    if (b.p) {
        cudaFreeAsync(b.p, m.s);
        b.p = nullptr;
        b.n = 0;
    }
    if (n == 0) return FE_OK;
    FE_CUDA(cudaMallocFromPoolAsync((void **)&b.p, n * sizeof(T), m.pool, m.s));
    b.n = n;
    return FE_OK;
}

template <typename T>
void pfree(const MgMem &m, DBuf<T> &b) {
    if (b.p) cudaFreeAsync(b.p, m.s);
    b.p = nullptr;
    b.n = 0;
}

inline void drelease(const MgMem &m, DevCsr &c) {
    pfree(m, c.ptr), pfree(m, c.col), pfree(m, c.val);
    c.nnzb = 0;
}

struct DevLevel {
    DevCsr A, P, PT;
    DBuf<double> dinv;
    DBuf<int32_t> agg;
    double lmax = 0.0;
    // the V-cycle runs in FP32: values of A, P, P^T and D^-1, and the level's vectors
    // (n * d each; r, x: the level's right-hand side and iterate)
    DBuf<float> a32, p32, pt32, dinv32;
    DBuf<float> r, x, t, dir, zn;
    void release(const MgMem &m) {
        drelease(m, A), drelease(m, P), drelease(m, PT);
        pfree(m, dinv), pfree(m, agg), pfree(m, a32), pfree(m, p32), pfree(m, pt32), pfree(m, dinv32);
        pfree(m, r), pfree(m, x), pfree(m, t), pfree(m, dir), pfree(m, zn);
    }
};

struct DevAmg {
    MgMem mem;                       // where every buffer below comes from
    std::vector<DevLevel> L;
    DevCsr coarse;
    int64_t nc = 0;                  // coarsest DOFs
    DBuf<double> cinv;               // dense inverse of the coarsest matrix (FP64)
    DBuf<float> rc, xc;
    int mis_rounds = 0;              // independent-set rounds, all levels
    ~DevAmg() {
        for (auto &l : L) l.release(mem);
        drelease(mem, coarse);
        pfree(mem, cinv), pfree(mem, rc), pfree(mem, xc);
    }
};

// Events recorded on the stream where each setup phase starts (amg::SetupPhase), while
// profiling: a phase runs from its mark to the next one.
struct SetupTrace {
    std::vector<std::pair<cudaEvent_t, int>> marks;
    void mark(cudaStream_t s, int k) {
        cudaEvent_t e = nullptr;
        if (cudaEventCreate(&e) != cudaSuccess) return;
        cudaEventRecord(e, s);
        marks.push_back({e, k});
    }
    // waits for the last mark, adds each phase's time to ms[k] (k < n)
    int collect(double *ms, int n) {
        if (marks.empty()) return FE_OK;
        FE_CUDA(cudaEventSynchronize(marks.back().first));
        for (size_t i = 0; i + 1 < marks.size(); ++i) {
            float a = 0.f;
            if (marks[i].second < n && cudaEventElapsedTime(&a, marks[i].first, marks[i + 1].first) == cudaSuccess)
                ms[marks[i].second] += a;
        }
        return FE_OK;
    }
    ~SetupTrace() {
        for (auto &m : marks) cudaEventDestroy(m.first);
    }
};

// Device setup of the hierarchy of the handle's eliminated system (near-null space: the
// rigid-body modes for elasticity, the constant for magnetostatics, zero on the
// constrained DOFs): amg::setup_hierarchy on the device executor; phases marked in
// trace when given.
int amg_setup_device(fe_handle_s *h, double theta, int64_t coarse_dofs, DevAmg &G, SetupTrace *trace = nullptr);
// Copy of a device hierarchy into host form (accessors of the fe_amg_* ABI).
int amg_download(const DevAmg &G, fe_amg_s *out, cudaStream_t s);
// Dense inverse of the coarsest matrix (+ 1e-12 of its largest diagonal entry).
int coarse_inverse_of(const BlockCsr &C, std::vector<double> &inv, const char *who);

}  // namespace fe
