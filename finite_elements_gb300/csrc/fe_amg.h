// Smoothed-aggregation hierarchy shared by its host setup (fe_amg_setup.cu) and the
// device cycle (fe_amg_device.cu).
#pragma once

#include <stdint.h>

#include <vector>

namespace fe {

struct BlockCsr {
    int64_t n = 0;             // block rows
    int rd = 0, cd = 0;        // block size rd x cd
    std::vector<int64_t> ptr;  // n + 1
    std::vector<int32_t> col;
    std::vector<double> val;   // nnzb * rd * cd, row-major blocks
    int64_t nnzb() const { return (int64_t)col.size(); }
};

struct AmgLevel {
    BlockCsr A;                 // d x d blocks
    BlockCsr P;                 // d x m blocks, columns = aggregates
    BlockCsr PT;                // m x d blocks: the restriction
    std::vector<double> dinv;   // block-diagonal pseudo-inverse of A
    std::vector<int32_t> agg;   // aggregate of each node
    double lmax = 0.0;
};

}  // namespace fe

struct fe_amg_s {
    std::vector<fe::AmgLevel> levels;
    fe::BlockCsr coarse;
    std::vector<double> coarse_inv;   // dense inverse of the coarsest matrix + 1e-12 max|diag| I
};
