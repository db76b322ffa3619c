// Learned warm start for PCG: a graph network over the mesh (nodes = mesh nodes,
// edges = the node pairs that share an element, i.e. the block pattern of K)
// predicts the shape u_hat of the displacement field; the warm start is
// x0 = g + s u_hat with g the prescribed values and s = (u_hat . b~) / (u_hat . A u_hat),
// the scale that minimises the A-norm error along u_hat (b~ = b - A g, zero on the
// constrained DOFs).  PCG from x0 to the same tolerance still decides the accuracy.
//
// Network (hidden width 64, 6 layers):
//   h0 = relu(f W0 + b0)                       f: 16 node features
//   m_l = mean_{j in N(i)} h_l,j               mesh-neighbour mean (no self)
//   g_l = mean_i h_l,i                         global mean
//   z_l = [h_l, m_l] W_l + b_l + g_l U_l
//   h_{l+1} = h_l + relu(z_l)
//   u_hat = (P S)^32 P (h_6 Wd + bd)          P: zero the constrained DOFs,
//                                              S = (I + mean_nbr) / 2 (low-pass)
// The fixed smoothing stage keeps u_hat smooth: in the A-norm a rough field is all
// energy and no overlap with the solution, so it would scale x0 to nothing.
// Loss: the share of the solution's energy the warm start leaves to PCG,
//   L = 1 - (u_hat . b~)^2 / ((u_hat . A u_hat) (b~ . v*)),  v* = u* - g,
// so training needs only b~ . v* from a solve of the problem.
//
// The dense transforms run as BF16 tcgen05 MMAs with FP32 accumulators in tensor
// memory, FP32 master weights and activations; aggregation, reductions,
// loss and Adam are FP32 / FP64 CUDA-core kernels.  Elasticity meshes only.
#include <cuda_bf16.h>
#include <math.h>
#include <stdint.h>
#include <string.h>

#include <algorithm>
#include <vector>

#include "fe_internal.h"

namespace fe {
namespace {

constexpr int HID = 64;
constexpr int NF = 16;
constexpr int NLAYER = 6;
constexpr int KC = 2 * HID;   // concatenated [h, m]
constexpr int NSMOOTH = 32;   // lazy neighbour-mean steps applied to the decoded field

// parameter offsets in the FP32 blob; every weight matrix is stored [in][out]
constexpr int P_W0 = 0;
constexpr int P_B0 = P_W0 + NF * HID;
constexpr int P_L0 = P_B0 + HID;
constexpr int L_W = 0;
constexpr int L_B = KC * HID;
constexpr int L_U = L_B + HID;
constexpr int L_STRIDE = L_U + HID * HID;
constexpr int P_WD = P_L0 + NLAYER * L_STRIDE;
constexpr int P_BD = P_WD + HID * 2;
constexpr int P_TOTAL = P_BD + 2;

constexpr int kT = 256;

inline int g1(int64_t n, int t = kT) { return grid_for(n, t, 152 * 8); }

// ---------------------------------------------------------------- tensor-core GEMMs
// The dense transforms on the 5th-generation tensor cores: BF16 x BF16 -> FP32
// tcgen05.mma (kind::f16, cta_group::1, M = 128) with the accumulator in tensor memory.
// Both operands are staged by the block's threads (the FP32 activations are rounded to
// BF16 on the way) into shared memory in the canonical K-major layout without swizzle:
// 8-row x 16-byte core matrices, element (r, k) of an R x K operand at byte
//   (r / 8) * (K * 16) + (k / 8) * 128 + (r % 8) * 16 + (k % 8) * 2,
// i.e. core matrices adjacent in K 128 bytes apart (the descriptor's leading byte
// offset) and 8-row groups K * 16 bytes apart (its stride byte offset).  One thread
// issues the K / 16 MMAs of a tile and commits them to an mbarrier; the eight warps then
// read the accumulator with tcgen05.ld for the epilogue, two warps per 32-lane quarter
// (a warp reaches only its quarter's lanes), each half of the columns.  Every wait
// is bounded: a wait that runs out sets *err, and the block frees its tensor memory
// and leaves.

constexpr int kTcRows = 128;                  // M of every MMA: rows of a tile
// Dynamic shared memory per block: 48 KB holds the operands of every shape and leaves
// at most 4 blocks (4 x 128 tensor-memory columns, the SM's 512) on an SM, so that an
// allocation of tensor memory never waits for another block.
constexpr size_t kTcSmem = 48 * 1024;
constexpr int kTcThreads = 256;   // 8 warps: two per 32-lane quarter of the accumulator
constexpr unsigned kTcSpin = 1u << 22;        // mbarrier polls (64 ns apart) before giving up

__device__ __forceinline__ uint32_t smem_addr(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }

// byte offset of element (r, k) of an operand with K columns in the canonical layout
__device__ __forceinline__ uint32_t tc_off(int r, int k, int K) {
    return (uint32_t)((r >> 3) * (K * 16) + (k >> 3) * 128 + (r & 7) * 16 + (k & 7) * 2);
}

// shared-memory matrix descriptor: start address, leading (K) and stride (8-row) byte
// offsets, version 1, no swizzle
__device__ __forceinline__ uint64_t tc_desc(uint32_t addr, uint32_t lbo, uint32_t sbo) {
    return (uint64_t)((addr & 0x3FFFFu) >> 4) | ((uint64_t)((lbo & 0x3FFFFu) >> 4) << 16) |
           ((uint64_t)((sbo & 0x3FFFFu) >> 4) << 32) | (1ull << 46);
}

// instruction descriptor of kind::f16: FP32 accumulator, BF16 A and B, both K-major
__host__ __device__ constexpr uint32_t tc_idesc(int m, int n) {
    return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(n >> 3) << 17) | ((uint32_t)(m >> 4) << 24);
}

__device__ __forceinline__ void tc_mma(uint32_t d_tmem, uint64_t a, uint64_t b, uint32_t idesc, uint32_t accumulate) {
    asm volatile(
        "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
        " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(d_tmem),
        "l"(a), "l"(b), "r"(idesc), "r"(accumulate));
}

__device__ __forceinline__ void tc_commit(uint64_t *mbar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_addr(mbar))
                 : "memory");
}

__device__ __forceinline__ void mbar_init(uint64_t *mbar) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_addr(mbar)) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

// waits for the phase with the given parity to complete; false after kTcSpin polls
__device__ __forceinline__ bool mbar_wait(uint64_t *mbar, uint32_t parity) {
    const uint32_t a = smem_addr(mbar);
    for (unsigned i = 0; i < kTcSpin; ++i) {
        uint32_t done;
        asm volatile(
            "{\n .reg .pred p;\n mbarrier.test_wait.parity.shared::cta.b64 p, [%1], %2;\n"
            " selp.u32 %0, 1, 0, p;\n}\n"
            : "=r"(done)
            : "r"(a), "r"(parity)
            : "memory");
        if (done) return true;
        __nanosleep(64);
    }
    return false;
}

__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void fence_async_smem() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

// warp 0: ncols tensor-memory columns, their address into *slot
__device__ __forceinline__ void tmem_alloc(uint32_t *slot, uint32_t ncols) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_addr(slot)),
                 "r"(ncols)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}

__device__ __forceinline__ void tmem_free(uint32_t taddr, uint32_t ncols) {
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols) : "memory");
}

// 16 consecutive FP32 columns of this thread's lane (the warp's 32 lanes from taddr)
__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float (&v)[16]) {
    uint32_t r[16];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
          "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
        : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
    for (int k = 0; k < 16; ++k) v[k] = __uint_as_float(r[k]);
}

__device__ __forceinline__ uint32_t pack_bf16(float lo, float hi) {
    return (uint32_t)__bfloat16_as_ushort(__float2bfloat16_rn(lo)) |
           ((uint32_t)__bfloat16_as_ushort(__float2bfloat16_rn(hi)) << 16);
}

enum Epi { EPI_RELU_BIAS = 0, EPI_LAYER = 1, EPI_PLAIN = 2 };

// Y[N x NO] = X[N x KI] W[KI x NO] (+ epilogue), X given as two row-major FP32 halves
// (columns [0, K1) from X1, [K1, KI) from X2), W given transposed in BF16 (Wt[n][k]).
// A tile: 128 rows of X (A, K-major) against all of Wt (B, K-major, staged once).
template <int KI, int K1, int NO, int EPI>
__global__ void __launch_bounds__(kTcThreads)
k_gemm(int64_t N, const float *__restrict__ X1, const float *__restrict__ X2, const __nv_bfloat16 *__restrict__ Wt,
       const float *__restrict__ bias, const float *__restrict__ gterm, const float *__restrict__ hres,
       float *__restrict__ Z, float *__restrict__ Y, int *err) {
    static_assert(KI % 16 == 0 && NO % 32 == 0 && NO <= 128 && K1 % 8 == 0, "tile shapes");
    constexpr uint32_t A_BYTES = kTcRows * KI * 2, NCOL = NO <= 64 ? 64 : 128;
    static_assert(A_BYTES + NO * KI * 2 <= 48 * 1024, "operands fit the block's shared memory");
    extern __shared__ __align__(1024) uint8_t smem[];
    uint8_t *As = smem, *Bs = smem + A_BYTES;
    __shared__ uint64_t mbar;
    __shared__ uint32_t tmem_slot;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    // B once: Wt[n][k], 16-byte chunks of 8 k
    for (int c = threadIdx.x; c < NO * KI / 8; c += blockDim.x) {
        const int n = c % NO, kc = c / NO;
        *reinterpret_cast<uint4 *>(Bs + tc_off(n, kc * 8, KI)) = *reinterpret_cast<const uint4 *>(Wt + n * KI + kc * 8);
    }
    if (threadIdx.x == 0) mbar_init(&mbar);
    if (warp == 0) tmem_alloc(&tmem_slot, NCOL);
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = tmem_slot;
    const uint64_t adesc = tc_desc(smem_addr(As), 128, KI * 16), bdesc = tc_desc(smem_addr(Bs), 128, KI * 16);
    constexpr uint32_t idesc = tc_idesc(kTcRows, NO);
    uint32_t phase = 0;
    bool ok = true;
    for (int64_t tile = blockIdx.x; tile * kTcRows < N && ok; tile += gridDim.x) {
        const int64_t row0 = tile * kTcRows;
        // A: 128 rows x KI, 16-byte chunks of 8 k (consecutive threads, consecutive rows);
        // a thread issues the loads of up to 4 chunks before it converts any of them, so
        // that 8 loads per thread are in flight
        constexpr int CHUNKS = kTcRows * KI / 8, PER = CHUNKS / kTcThreads, BATCH = PER < 4 ? PER : 4;
        static_assert(CHUNKS % kTcThreads == 0 && PER % BATCH == 0, "chunks per thread");
#pragma unroll
        for (int j0 = 0; j0 < PER; j0 += BATCH) {
            float4 v[BATCH][2];
#pragma unroll
            for (int j = 0; j < BATCH; ++j) {
                const int c = threadIdx.x + (j0 + j) * kTcThreads;
                const int r = c % kTcRows, k = (c / kTcRows) * 8;
                const int64_t gr = row0 + r;
                v[j][0] = v[j][1] = make_float4(0.f, 0.f, 0.f, 0.f);
                if (gr < N) {
                    const float *src = k < K1 ? X1 + gr * K1 + k : X2 + gr * (KI - K1) + (k - K1);
                    v[j][0] = *reinterpret_cast<const float4 *>(src);
                    v[j][1] = *reinterpret_cast<const float4 *>(src + 4);
                }
            }
#pragma unroll
            for (int j = 0; j < BATCH; ++j) {
                const int c = threadIdx.x + (j0 + j) * kTcThreads;
                const int r = c % kTcRows, k = (c / kTcRows) * 8;
                uint4 q;
                q.x = pack_bf16(v[j][0].x, v[j][0].y), q.y = pack_bf16(v[j][0].z, v[j][0].w);
                q.z = pack_bf16(v[j][1].x, v[j][1].y), q.w = pack_bf16(v[j][1].z, v[j][1].w);
                *reinterpret_cast<uint4 *>(As + tc_off(r, k, KI)) = q;
            }
        }
        fence_async_smem();
        __syncthreads();
        if (threadIdx.x == 0) {
            tc_fence_after();
#pragma unroll
            for (int kk = 0; kk < KI; kk += 16)   // K = 16: two core matrices, 256 bytes (16 units) on
                tc_mma(tmem, adesc + (uint64_t)kk, bdesc + (uint64_t)kk, idesc, kk > 0);
            tc_commit(&mbar);
        }
        ok = __syncthreads_and(mbar_wait(&mbar, phase));   // the same outcome in every thread
        phase ^= 1;
        tc_fence_after();
        if (ok) {
            // warp w: accumulator lanes (rows) 32 (w % 4) .., columns of half w / 4
            const int quarter = warp & 3, half = warp >> 2;
            const int64_t r = row0 + quarter * 32 + lane;
#pragma unroll
            for (int c0 = half * (NO / 2); c0 < (half + 1) * (NO / 2); c0 += 16) {
                float v[16];
                tmem_ld16(tmem + ((uint32_t)(quarter * 32) << 16) + (uint32_t)c0, v);
                if (r < N) {
#pragma unroll
                    for (int q = 0; q < 16; q += 4) {
                        const int c = c0 + q;
                        float4 o = make_float4(v[q], v[q + 1], v[q + 2], v[q + 3]);
                        if (EPI == EPI_PLAIN) {
                            *reinterpret_cast<float4 *>(Y + r * NO + c) = o;
                        } else {
                            o.x += bias[c], o.y += bias[c + 1], o.z += bias[c + 2], o.w += bias[c + 3];
                            if (EPI == EPI_LAYER)
                                o.x += gterm[c], o.y += gterm[c + 1], o.z += gterm[c + 2], o.w += gterm[c + 3];
                            *reinterpret_cast<float4 *>(Z + r * NO + c) = o;
                            float4 y = make_float4(fmaxf(o.x, 0.f), fmaxf(o.y, 0.f), fmaxf(o.z, 0.f), fmaxf(o.w, 0.f));
                            if (EPI == EPI_LAYER) {
                                const float4 h = *reinterpret_cast<const float4 *>(hres + r * NO + c);
                                y.x += h.x, y.y += h.y, y.z += h.z, y.w += h.w;
                            }
                            *reinterpret_cast<float4 *>(Y + r * NO + c) = y;
                        }
                    }
                }
            }
        } else if (threadIdx.x == 0) {
            atomicExch(err, 1);
        }
        tc_fence_before();
        __syncthreads();
    }
    tc_fence_after();
    if (warp == 0) tmem_free(tmem, NCOL);
}

// dW[KI x NO] += X^T dZ over all rows (X given as two FP32 halves as above, dZ [N x NO]):
// C (128 x NO) = A B^T with A = X^T (rows of features, zero past KI) and B = dZ^T, both
// K-major with K = 128 rows of the mesh per tile, accumulated in tensor memory over the
// block's tiles; each block adds its partial dW with FP32 atomics at the end.
template <int KI, int K1, int NO>
__global__ void __launch_bounds__(kTcThreads)
k_gemm_wgrad(int64_t N, const float *__restrict__ X1, const float *__restrict__ X2, const float *__restrict__ dZ,
             float *__restrict__ dW, int *err) {
    static_assert(KI <= 128 && KI % 16 == 0 && NO % 32 == 0 && NO <= 128 && K1 % 2 == 0, "tile shapes");
    constexpr int KT = kTcRows;   // rows of the mesh per tile (the MMA's K)
    constexpr uint32_t A_BYTES = 128 * KT * 2, NCOL = NO <= 64 ? 64 : 128;
    static_assert(A_BYTES + NO * KT * 2 <= 48 * 1024, "operands fit the block's shared memory");
    extern __shared__ __align__(1024) uint8_t smem[];
    uint8_t *As = smem, *Bs = smem + A_BYTES;
    __shared__ uint64_t mbar;
    __shared__ uint32_t tmem_slot;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    // feature rows past KI stay zero
    for (int i = threadIdx.x; i < (int)(A_BYTES / 16); i += blockDim.x)
        reinterpret_cast<uint4 *>(As)[i] = make_uint4(0u, 0u, 0u, 0u);
    if (threadIdx.x == 0) mbar_init(&mbar);
    if (warp == 0) tmem_alloc(&tmem_slot, NCOL);
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = tmem_slot;
    const uint64_t adesc = tc_desc(smem_addr(As), 128, KT * 16), bdesc = tc_desc(smem_addr(Bs), 128, KT * 16);
    constexpr uint32_t idesc = tc_idesc(128, NO);
    uint32_t phase = 0, used = 0;
    bool ok = true;
    for (int64_t tile = blockIdx.x; tile * KT < N && ok; tile += gridDim.x) {
        const int64_t row0 = tile * KT;
        // a thread packs 8 consecutive mesh rows of one feature pair into two 16-byte chunks
        for (int c = threadIdx.x; c < (KI / 2) * (KT / 8); c += blockDim.x) {
            const int fp = c % (KI / 2), kg = c / (KI / 2);
            const int m = 2 * fp;
            float a0[8], a1[8];
#pragma unroll
            for (int q = 0; q < 8; ++q) {
                const int64_t gr = row0 + kg * 8 + q;
                float2 v = make_float2(0.f, 0.f);
                if (gr < N)
                    v = m < K1 ? *reinterpret_cast<const float2 *>(X1 + gr * K1 + m)
                               : *reinterpret_cast<const float2 *>(X2 + gr * (KI - K1) + (m - K1));
                a0[q] = v.x, a1[q] = v.y;
            }
            *reinterpret_cast<uint4 *>(As + tc_off(m, kg * 8, KT)) =
                make_uint4(pack_bf16(a0[0], a0[1]), pack_bf16(a0[2], a0[3]), pack_bf16(a0[4], a0[5]),
                           pack_bf16(a0[6], a0[7]));
            *reinterpret_cast<uint4 *>(As + tc_off(m + 1, kg * 8, KT)) =
                make_uint4(pack_bf16(a1[0], a1[1]), pack_bf16(a1[2], a1[3]), pack_bf16(a1[4], a1[5]),
                           pack_bf16(a1[6], a1[7]));
        }
        for (int c = threadIdx.x; c < (NO / 2) * (KT / 8); c += blockDim.x) {
            const int np = c % (NO / 2), kg = c / (NO / 2);
            const int n = 2 * np;
            float b0[8], b1[8];
#pragma unroll
            for (int q = 0; q < 8; ++q) {
                const int64_t gr = row0 + kg * 8 + q;
                const float2 v = gr < N ? *reinterpret_cast<const float2 *>(dZ + gr * NO + n) : make_float2(0.f, 0.f);
                b0[q] = v.x, b1[q] = v.y;
            }
            *reinterpret_cast<uint4 *>(Bs + tc_off(n, kg * 8, KT)) =
                make_uint4(pack_bf16(b0[0], b0[1]), pack_bf16(b0[2], b0[3]), pack_bf16(b0[4], b0[5]),
                           pack_bf16(b0[6], b0[7]));
            *reinterpret_cast<uint4 *>(Bs + tc_off(n + 1, kg * 8, KT)) =
                make_uint4(pack_bf16(b1[0], b1[1]), pack_bf16(b1[2], b1[3]), pack_bf16(b1[4], b1[5]),
                           pack_bf16(b1[6], b1[7]));
        }
        fence_async_smem();
        __syncthreads();
        if (threadIdx.x == 0) {
            tc_fence_after();
#pragma unroll
            for (int kk = 0; kk < KT; kk += 16)
                tc_mma(tmem, adesc + (uint64_t)kk, bdesc + (uint64_t)kk, idesc, (used | kk) != 0);
            tc_commit(&mbar);
        }
        used = 1;
        // the MMAs read the staged tiles: wait before they are overwritten
        ok = __syncthreads_and(mbar_wait(&mbar, phase));
        phase ^= 1;
        tc_fence_after();
    }
    if (!ok) {
        if (threadIdx.x == 0) atomicExch(err, 1);
    } else if (used && (warp & 3) * 32 < KI) {
        const int quarter = warp & 3, half = warp >> 2;
        const int m = quarter * 32 + lane;
#pragma unroll
        for (int c0 = half * (NO / 2); c0 < (half + 1) * (NO / 2); c0 += 16) {
            float v[16];
            tmem_ld16(tmem + ((uint32_t)(quarter * 32) << 16) + (uint32_t)c0, v);
            if (m < KI)
#pragma unroll
                for (int q = 0; q < 16; ++q) atomicAdd(&dW[m * NO + c0 + q], v[q]);
        }
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    if (warp == 0) tmem_free(tmem, NCOL);
}

// ---------------------------------------------------------------- graph kernels

// m_r = inv_deg[r] * sum_{c in N(r), c != r} h_c   (TRANSPOSE: out_c += sum inv_deg[r] h_r)
// one warp per node, two features per lane.
template <bool TRANSPOSE>
__global__ void k_aggregate(int64_t n, const int32_t *__restrict__ ptr, const int32_t *__restrict__ col,
                            const float *__restrict__ inv_deg, const float *__restrict__ hin, float *__restrict__ out) {
    const int lane = threadIdx.x & 31;
    const int64_t warps = ((int64_t)gridDim.x * blockDim.x) >> 5;
    for (int64_t r = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; r < n; r += warps) {
        float2 acc = make_float2(0.f, 0.f);
        for (int s = ptr[r]; s < ptr[r + 1]; ++s) {
            const int c = col[s];
            if (c == (int)r) continue;
            const float w = TRANSPOSE ? inv_deg[c] : 1.f;
            const float2 v = reinterpret_cast<const float2 *>(hin + (int64_t)c * HID)[lane];
            acc.x += w * v.x;
            acc.y += w * v.y;
        }
        float2 *o = reinterpret_cast<float2 *>(out + r * HID) + lane;
        if (TRANSPOSE) {
            float2 cur = *o;
            *o = make_float2(cur.x + acc.x, cur.y + acc.y);
        } else {
            const float w = inv_deg[r];
            *o = make_float2(acc.x * w, acc.y * w);
        }
    }
}

__global__ void k_inv_deg(int64_t n, const int32_t *__restrict__ ptr, const int32_t *__restrict__ col,
                          float *__restrict__ inv_deg) {
    for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < n; r += (int64_t)gridDim.x * blockDim.x) {
        int d = 0;
        for (int s = ptr[r]; s < ptr[r + 1]; ++s) d += col[s] != (int)r;
        inv_deg[r] = d > 0 ? 1.f / (float)d : 0.f;
    }
}

// out[64] += column sums of X [n x 64] (out zeroed by the caller)
__global__ void k_colsum(int64_t n, const float *__restrict__ X, float *__restrict__ out) {
    __shared__ float sh[kT / 64][64];
    const int c = threadIdx.x & 63, rg = threadIdx.x >> 6;   // 4 row groups of 64 columns
    float acc = 0.f;
    for (int64_t r = (int64_t)blockIdx.x * (kT / 64) + rg; r < n; r += (int64_t)gridDim.x * (kT / 64))
        acc += X[r * HID + c];
    sh[rg][c] = acc;
    __syncthreads();
    if (rg == 0) {
        float s = sh[0][c] + sh[1][c] + sh[2][c] + sh[3][c];
        atomicAdd(&out[c], s);
    }
}

// gterm[n] = sum_k (colsum[k] / N) U[k][n]     (one block of 64 threads)
__global__ void k_gterm(const float *__restrict__ colsum, float inv_n, const float *__restrict__ U,
                        float *__restrict__ gterm) {
    const int c = threadIdx.x;
    float acc = 0.f;
    for (int k = 0; k < HID; ++k) acc += colsum[k] * inv_n * U[k * HID + c];
    gterm[c] = acc;
}

// dZ = dH (.) [z > 0]
__global__ void k_relu_grad(int64_t n, const float *__restrict__ dH, const float *__restrict__ Z,
                            float *__restrict__ dZ) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        dZ[i] = Z[i] > 0.f ? dH[i] : 0.f;
}

// dH[:, :] = dH_next + dX[:, :64] + dgb (broadcast)     (dX is [n x 128])
__global__ void k_layer_back_dh(int64_t n, const float *__restrict__ dHn, const float *__restrict__ dX,
                                const float *__restrict__ dgb, float *__restrict__ dH) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n * HID;
         i += (int64_t)gridDim.x * blockDim.x) {
        int64_t r = i / HID;
        int c = (int)(i - r * HID);
        dH[i] = dHn[i] + dX[r * KC + c] + dgb[c];
    }
}

// dM = dX[:, 64:]
__global__ void k_split_dm(int64_t n, const float *__restrict__ dX, float *__restrict__ dM) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n * HID;
         i += (int64_t)gridDim.x * blockDim.x) {
        int64_t r = i / HID;
        int c = (int)(i - r * HID);
        dM[i] = dX[r * KC + HID + c];
    }
}

// global-term gradients from s = colsum(dZ): dU[k][n] += g[k] s[n], dgb[k] = (1/N) sum_n U[k][n] s[n]
__global__ void k_gterm_back(const float *__restrict__ colsum_h, float inv_n, const float *__restrict__ U,
                             const float *__restrict__ s, float *__restrict__ dU, float *__restrict__ dgb) {
    const int k = threadIdx.x;
    const float gk = colsum_h[k] * inv_n;
    float acc = 0.f;
    for (int c = 0; c < HID; ++c) {
        dU[k * HID + c] += gk * s[c];
        acc += U[k * HID + c] * s[c];
    }
    dgb[k] = acc * inv_n;
}

// ---------------------------------------------------------------- features, decoder, loss

struct Bounds {
    float xmin, xmax, ymin, ymax;
};

__device__ __forceinline__ void atomic_min_f(float *addr, float v) {
    int old = __float_as_int(*addr);
    while (__int_as_float(old) > v) {
        int prev = atomicCAS(reinterpret_cast<int *>(addr), old, __float_as_int(v));
        if (prev == old) break;
        old = prev;
    }
}
__device__ __forceinline__ void atomic_max_f(float *addr, float v) {
    int old = __float_as_int(*addr);
    while (__int_as_float(old) < v) {
        int prev = atomicCAS(reinterpret_cast<int *>(addr), old, __float_as_int(v));
        if (prev == old) break;
        old = prev;
    }
}

// stats[0..3] = bounding box (FP32 atomics)
__global__ void k_bbox(int64_t n, const double *__restrict__ coords, float *__restrict__ stats) {
    float xmn = 3.4e38f, xmx = -3.4e38f, ymn = 3.4e38f, ymx = -3.4e38f;
    for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < n; r += (int64_t)gridDim.x * blockDim.x) {
        float x = (float)coords[2 * r], y = (float)coords[2 * r + 1];
        xmn = fminf(xmn, x), xmx = fmaxf(xmx, x), ymn = fminf(ymn, y), ymx = fmaxf(ymx, y);
    }
    for (int o = 16; o > 0; o >>= 1) {
        xmn = fminf(xmn, __shfl_xor_sync(0xffffffffu, xmn, o));
        xmx = fmaxf(xmx, __shfl_xor_sync(0xffffffffu, xmx, o));
        ymn = fminf(ymn, __shfl_xor_sync(0xffffffffu, ymn, o));
        ymx = fmaxf(ymx, __shfl_xor_sync(0xffffffffu, ymx, o));
    }
    if ((threadIdx.x & 31) == 0) {
        atomic_min_f(&stats[0], xmn);
        atomic_max_f(&stats[1], xmx);
        atomic_min_f(&stats[2], ymn);
        atomic_max_f(&stats[3], ymx);
    }
}

// Graph-level load moments (FP64 atomics): gs[0] += sum b~_x, gs[1] += sum b~_y,
// gs[2] += sum |b~|, gs[3] += sum b~_y x_n, gs[4] += sum b~_x y_n   (normalised
// coordinates from the bounding box in stats)
__global__ void k_load_moments(int64_t n, const double *__restrict__ coords, const double *__restrict__ bt,
                               const float *__restrict__ stats, double *__restrict__ gs) {
    const double L = fmax(fmax((double)stats[1] - stats[0], (double)stats[3] - stats[2]), 1e-30);
    double a[5] = {0, 0, 0, 0, 0};
    for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < n; r += (int64_t)gridDim.x * blockDim.x) {
        const double xn = (coords[2 * r] - stats[0]) / L, yn = (coords[2 * r + 1] - stats[2]) / L;
        const double bx = bt[2 * r], by = bt[2 * r + 1];
        a[0] += bx, a[1] += by, a[2] += fabs(bx) + fabs(by), a[3] += by * xn, a[4] += bx * yn;
    }
#pragma unroll
    for (int k = 0; k < 5; ++k) {
        for (int o = 16; o > 0; o >>= 1) a[k] += __shfl_xor_sync(0xffffffffu, a[k], o);
        if ((threadIdx.x & 31) == 0) atomicAdd(&gs[k], a[k]);
    }
}

// Graph-level material means: gs[5] += sum log10 E, gs[6] += sum nu over the elements
__global__ void k_material_means(int64_t ne, const double *__restrict__ E, const double *__restrict__ nu,
                                 double *__restrict__ gs) {
    double a = 0, b = 0;
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < ne; e += (int64_t)gridDim.x * blockDim.x)
        a += log10(E[e]), b += nu[e];
    for (int o = 16; o > 0; o >>= 1) {
        a += __shfl_xor_sync(0xffffffffu, a, o);
        b += __shfl_xor_sync(0xffffffffu, b, o);
    }
    if ((threadIdx.x & 31) == 0) {
        atomicAdd(&gs[5], a);
        atomicAdd(&gs[6], b);
    }
}

// 16 features per node: smooth per-node inputs (position, Fourier terms, constraint
// flags) and graph-level quantities broadcast to every node (total-force direction,
// load moments, mean log10 E and nu).  No per-node load or material value: those
// vary from node to node and would make the network's output rough.
__global__ void k_features(int64_t n, int64_t ne, const double *__restrict__ coords,
                           const int32_t *__restrict__ bc_of_dof, const float *__restrict__ stats,
                           const double *__restrict__ gs, float *__restrict__ F) {
    const float L = fmaxf(fmaxf(stats[1] - stats[0], stats[3] - stats[2]), 1e-30f);
    const double fn = sqrt(gs[0] * gs[0] + gs[1] * gs[1]);
    const float fx = fn > 0 ? (float)(gs[0] / fn) : 0.f, fy = fn > 0 ? (float)(gs[1] / fn) : 0.f;
    const float m1 = gs[2] > 0 ? (float)(gs[3] / gs[2]) : 0.f, m2 = gs[2] > 0 ? (float)(gs[4] / gs[2]) : 0.f;
    const float le = ne > 0 ? (float)(gs[5] / ne) - 10.5f : 0.f, lnu = ne > 0 ? ((float)(gs[6] / ne) - 0.3f) * 10.f : 0.f;
    const float PI = 3.14159265358979f;
    for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < n; r += (int64_t)gridDim.x * blockDim.x) {
        float xn = ((float)coords[2 * r] - stats[0]) / L, yn = ((float)coords[2 * r + 1] - stats[2]) / L;
        float *f = F + r * NF;
        f[0] = xn;
        f[1] = yn;
        f[2] = sinf(PI * xn);
        f[3] = cosf(PI * xn);
        f[4] = sinf(PI * yn);
        f[5] = cosf(PI * yn);
        f[6] = sinf(2.f * PI * xn);
        f[7] = sinf(2.f * PI * yn);
        f[8] = bc_of_dof[2 * r] >= 0 ? 1.f : 0.f;
        f[9] = bc_of_dof[2 * r + 1] >= 0 ? 1.f : 0.f;
        f[10] = fx;
        f[11] = fy;
        f[12] = m1;
        f[13] = m2;
        f[14] = le;
        f[15] = lnu;
    }
}

// g_ext (prescribed values on constrained DOFs, 0 elsewhere)
__global__ void k_gext(int64_t n_bc, const int64_t *__restrict__ bc_dof, const double *__restrict__ bc_val,
                       double *__restrict__ g) {
    for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < n_bc; k += (int64_t)gridDim.x * blockDim.x)
        g[bc_dof[k]] = bc_val[k];
}

// b~ = b - A g on free DOFs, 0 on constrained ones (Ag holds A g)
__global__ void k_btilde(int64_t n_dof, const double *__restrict__ b, const double *__restrict__ Ag,
                         const int32_t *__restrict__ bc_of_dof, double *__restrict__ bt) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n_dof; i += (int64_t)gridDim.x * blockDim.x)
        bt[i] = bc_of_dof[i] >= 0 ? 0.0 : b[i] - Ag[i];
}

// u_i = h_i Wd + bd (two outputs), zero on constrained DOFs; one warp per node
__global__ void k_decode(int64_t n, const float *__restrict__ Hh, const float *__restrict__ Wd,
                         const float *__restrict__ bd, const int32_t *__restrict__ bc_of_dof, float *__restrict__ u) {
    const int lane = threadIdx.x & 31;
    const int64_t warps = ((int64_t)gridDim.x * blockDim.x) >> 5;
    for (int64_t r = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; r < n; r += warps) {
        float2 h = reinterpret_cast<const float2 *>(Hh + r * HID)[lane];
        int k = 2 * lane;
        float o0 = h.x * Wd[k * 2] + h.y * Wd[(k + 1) * 2];
        float o1 = h.x * Wd[k * 2 + 1] + h.y * Wd[(k + 1) * 2 + 1];
        for (int o = 16; o > 0; o >>= 1) {
            o0 += __shfl_xor_sync(0xffffffffu, o0, o);
            o1 += __shfl_xor_sync(0xffffffffu, o1, o);
        }
        if (lane == 0) {
            u[2 * r] = bc_of_dof[2 * r] >= 0 ? 0.f : o0 + bd[0];
            u[2 * r + 1] = bc_of_dof[2 * r + 1] >= 0 ? 0.f : o1 + bd[1];
        }
    }
}

// One step of the smoothing stage on the two-component node field:
//   forward  (TRANSPOSE = false): out = P S in,   S = (I + mean_nbr) / 2
//   adjoint  (TRANSPOSE = true):  out = S^T P in, S^T = (I + mean_nbr^T) / 2
// mean_nbr^T gathers in[c] inv_deg[c] over the neighbours c of r (symmetric pattern).
template <bool TRANSPOSE>
__global__ void k_smooth(int64_t n, const int32_t *__restrict__ ptr, const int32_t *__restrict__ col,
                         const float *__restrict__ inv_deg, const int32_t *__restrict__ bc_of_dof,
                         const float *__restrict__ in, float *__restrict__ out) {
    for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < n; r += (int64_t)gridDim.x * blockDim.x) {
        float a0 = 0.f, a1 = 0.f;
        for (int s = ptr[r]; s < ptr[r + 1]; ++s) {
            const int c = col[s];
            if (c == (int)r) continue;
            float v0 = in[2 * (int64_t)c], v1 = in[2 * (int64_t)c + 1];
            if (TRANSPOSE) {
                const float w = inv_deg[c];
                v0 = bc_of_dof[2 * (int64_t)c] >= 0 ? 0.f : v0 * w;
                v1 = bc_of_dof[2 * (int64_t)c + 1] >= 0 ? 0.f : v1 * w;
            }
            a0 += v0;
            a1 += v1;
        }
        float s0 = in[2 * r], s1 = in[2 * r + 1];
        if (TRANSPOSE) {
            if (bc_of_dof[2 * r] >= 0) s0 = 0.f;
            if (bc_of_dof[2 * r + 1] >= 0) s1 = 0.f;
            out[2 * r] = 0.5f * (s0 + a0);
            out[2 * r + 1] = 0.5f * (s1 + a1);
        } else {
            const float w = inv_deg[r];
            out[2 * r] = bc_of_dof[2 * r] >= 0 ? 0.f : 0.5f * (s0 + w * a0);
            out[2 * r + 1] = bc_of_dof[2 * r + 1] >= 0 ? 0.f : 0.5f * (s1 + w * a1);
        }
    }
}

__global__ void k_f32_to_f64(int64_t n, const float *__restrict__ a, double *__restrict__ b) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        b[i] = (double)a[i];
}

// zero the constrained DOFs of a two-component field
__global__ void k_mask2(int64_t n_dof, const int32_t *__restrict__ bc_of_dof, float *__restrict__ v) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n_dof; i += (int64_t)gridDim.x * blockDim.x)
        if (bc_of_dof[i] >= 0) v[i] = 0.f;
}

// acc[0] += u.bt, acc[1] += u.Au  (FP64, block partials then atomics)
__global__ void k_dots2(int64_t n, const double *__restrict__ u, const double *__restrict__ bt,
                        const double *__restrict__ Au, double *__restrict__ acc) {
    __shared__ double sh[2][kT / 32];
    double s0 = 0, s1 = 0;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        s0 += u[i] * bt[i];
        s1 += u[i] * Au[i];
    }
    for (int o = 16; o > 0; o >>= 1) {
        s0 += __shfl_xor_sync(0xffffffffu, s0, o);
        s1 += __shfl_xor_sync(0xffffffffu, s1, o);
    }
    if ((threadIdx.x & 31) == 0) sh[0][threadIdx.x >> 5] = s0, sh[1][threadIdx.x >> 5] = s1;
    __syncthreads();
    if (threadIdx.x == 0) {
        double a = 0, c = 0;
        for (int w = 0; w < kT / 32; ++w) a += sh[0][w], c += sh[1][w];
        atomicAdd(&acc[0], a);
        atomicAdd(&acc[1], c);
    }
}

// du = ca * bt + cb * Au on free DOFs (0 on constrained), as FP32 per node pair
__global__ void k_loss_grad_u(int64_t n_dof, const double *__restrict__ bt, const double *__restrict__ Au,
                              const int32_t *__restrict__ bc_of_dof, double ca, double cb, float *__restrict__ du) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n_dof; i += (int64_t)gridDim.x * blockDim.x)
        du[i] = bc_of_dof[i] >= 0 ? 0.f : (float)(ca * bt[i] + cb * Au[i]);
}

// decoder backward: dH_i = Wd du_i; dWd += h_i du_i^T; dbd += du_i.  One warp per node.
__global__ void k_decode_back(int64_t n, const float *__restrict__ Hh, const float *__restrict__ Wd,
                              const float *__restrict__ du, float *__restrict__ dH, float *__restrict__ dWd,
                              float *__restrict__ dbd) {
    const int lane = threadIdx.x & 31;
    const int64_t warps = ((int64_t)gridDim.x * blockDim.x) >> 5;
    float w00 = 0, w01 = 0, w10 = 0, w11 = 0, b0 = 0, b1 = 0;
    const int k = 2 * lane;
    for (int64_t r = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; r < n; r += warps) {
        const float d0 = du[2 * r], d1 = du[2 * r + 1];
        float2 h = reinterpret_cast<const float2 *>(Hh + r * HID)[lane];
        reinterpret_cast<float2 *>(dH + r * HID)[lane] =
            make_float2(Wd[k * 2] * d0 + Wd[k * 2 + 1] * d1, Wd[(k + 1) * 2] * d0 + Wd[(k + 1) * 2 + 1] * d1);
        w00 += h.x * d0, w01 += h.x * d1, w10 += h.y * d0, w11 += h.y * d1;
        if (lane == 0) b0 += d0, b1 += d1;
    }
    atomicAdd(&dWd[k * 2], w00);
    atomicAdd(&dWd[k * 2 + 1], w01);
    atomicAdd(&dWd[(k + 1) * 2], w10);
    atomicAdd(&dWd[(k + 1) * 2 + 1], w11);
    if (lane == 0) {
        atomicAdd(&dbd[0], b0);
        atomicAdd(&dbd[1], b1);
    }
}

// Fitting loss against a solution x: t = (x - g) / sigma on free DOFs, sigma the RMS
// of x - g over them.  Pass 1: acc[0] += sum (x - g)^2 and acc[1] += free count over the
// free DOFs.  Pass 2 (sigma, n_free known): du = 2 (u - t) / n_free, acc[2] += (u - t)^2.
__global__ void k_fit_stats(int64_t n_dof, const double *__restrict__ x, const double *__restrict__ g,
                            const int32_t *__restrict__ bc_of_dof, double *__restrict__ acc) {
    __shared__ double sh[2][kT / 32];
    double s0 = 0, s1 = 0;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n_dof; i += (int64_t)gridDim.x * blockDim.x)
        if (bc_of_dof[i] < 0) {
            double d = x[i] - g[i];
            s0 += d * d;
            s1 += 1.0;
        }
    for (int o = 16; o > 0; o >>= 1) {
        s0 += __shfl_xor_sync(0xffffffffu, s0, o);
        s1 += __shfl_xor_sync(0xffffffffu, s1, o);
    }
    if ((threadIdx.x & 31) == 0) sh[0][threadIdx.x >> 5] = s0, sh[1][threadIdx.x >> 5] = s1;
    __syncthreads();
    if (threadIdx.x == 0) {
        double a = 0, c = 0;
        for (int w = 0; w < kT / 32; ++w) a += sh[0][w], c += sh[1][w];
        atomicAdd(&acc[0], a);
        atomicAdd(&acc[1], c);
    }
}

__global__ void k_fit_grad(int64_t n_dof, const double *__restrict__ u, const double *__restrict__ x,
                           const double *__restrict__ g, const int32_t *__restrict__ bc_of_dof, double inv_sigma,
                           double inv_n, float *__restrict__ du, double *__restrict__ acc) {
    __shared__ double sh[kT / 32];
    double s0 = 0;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n_dof; i += (int64_t)gridDim.x * blockDim.x) {
        if (bc_of_dof[i] >= 0) {
            du[i] = 0.f;
            continue;
        }
        double e = u[i] - (x[i] - g[i]) * inv_sigma;
        du[i] = (float)(2.0 * e * inv_n);
        s0 += e * e;
    }
    for (int o = 16; o > 0; o >>= 1) s0 += __shfl_xor_sync(0xffffffffu, s0, o);
    if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = s0;
    __syncthreads();
    if (threadIdx.x == 0) {
        double a = 0;
        for (int w = 0; w < kT / 32; ++w) a += sh[w];
        atomicAdd(acc, a);
    }
}

// x0 = g_ext + s u_hat
__global__ void k_warm_start(int64_t n_dof, const double *__restrict__ g, const double *__restrict__ u, double s,
                             double *__restrict__ x0) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n_dof; i += (int64_t)gridDim.x * blockDim.x)
        x0[i] = g[i] + s * u[i];
}

// the same with s = (u.b~) / (u.A u) from the device sums acc[0], acc[1] (0 when the
// denominator is not positive), for predictions that do not wait for the host
__global__ void k_warm_start_dev(int64_t n_dof, const double *__restrict__ g, const double *__restrict__ u,
                                 const double *__restrict__ acc, double *__restrict__ x0) {
    const double den = acc[1];
    const double s = den > 0 ? acc[0] / den : 0.0;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n_dof; i += (int64_t)gridDim.x * blockDim.x)
        x0[i] = g[i] + s * u[i];
}

// the bounding-box and moment accumulators' starting values
__global__ void k_init_stats(float *stats) {
    const float init[8] = {3.4e38f, -3.4e38f, 3.4e38f, -3.4e38f, 0.f, 0.f, 0.f, 0.f};
    if (threadIdx.x < 8) stats[threadIdx.x] = init[threadIdx.x];
}

// e = b~ . (x - g)   (energy of the solution's free part: b~ = A v* with v* = x - g)
__global__ void k_energy(int64_t n_dof, const double *__restrict__ bt, const double *__restrict__ x,
                         const double *__restrict__ g, double *__restrict__ acc) {
    __shared__ double sh[kT / 32];
    double s = 0;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n_dof; i += (int64_t)gridDim.x * blockDim.x)
        s += bt[i] * (x[i] - g[i]);
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x == 0) {
        double a = 0;
        for (int w = 0; w < kT / 32; ++w) a += sh[w];
        atomicAdd(acc, a);
    }
}

// W [KI][NO] FP32 -> Wt [NO][KI] BF16
__global__ void k_to_bf16_t(const float *__restrict__ W, int KI, int NO, __nv_bfloat16 *__restrict__ Wt) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < KI * NO; i += gridDim.x * blockDim.x) {
        int n = i / KI, k = i - n * KI;
        Wt[i] = __float2bfloat16_rn(W[k * NO + n]);
    }
}

// W FP32 -> BF16, same layout
__global__ void k_to_bf16(const float *__restrict__ W, int n, __nv_bfloat16 *__restrict__ out) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
        out[i] = __float2bfloat16_rn(W[i]);
}

// Adam on the FP32 master weights
__global__ void k_adam(int n, float *__restrict__ p, const float *__restrict__ gr, float *__restrict__ m,
                       float *__restrict__ v, float lr, float b1, float b2, float eps, float c1, float c2) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        float gi = gr[i];
        float mi = b1 * m[i] + (1.f - b1) * gi;
        float vi = b2 * v[i] + (1.f - b2) * gi * gi;
        m[i] = mi;
        v[i] = vi;
        p[i] -= lr * (mi / c1) / (sqrtf(vi / c2) + eps);
    }
}

}  // namespace
}  // namespace fe

// ---------------------------------------------------------------- network state

struct fe_gnn_s {
    fe::DBuf<float> params, grad, adam_m, adam_v;
    fe::DBuf<__nv_bfloat16> wt;   // transposed BF16 copies of W0, W_l (in that order)
    int64_t n_cap = 0;            // nodes the activation buffers hold
    fe::DBuf<float> F, Z0, H, Z, M, dH, dHn, dX, dZ, dM, inv_deg, colsum, gterm, stats, du, dgb;
    fe::DBuf<float> us0, us1;     // decoded field and the smoothing ping-pong buffer
    fe::DBuf<double> gext, Ag, bt, u, Au, x0, acc, gsum;
    fe::DBuf<int> tc_err;         // set by a tensor-core GEMM whose MMAs did not complete
    // asynchronous predictions run on the network's own stream, after `assembled` (the
    // handle's stream at the call) and until `ready` (which the handle's next solve waits on)
    cudaStream_t own = nullptr;
    cudaEvent_t assembled = nullptr, ready = nullptr;
    double *acc_host = nullptr;
    int steps = 0;
    double last_scale = 0.0, last_num = 0.0, last_den = 0.0;
    // stream of the handle the current call works on; valid only during that call
    // (a handle and its stream may be destroyed before the network)
    cudaStream_t stream = nullptr;
};

namespace fe {
namespace {

constexpr int WT_W0 = 0;
constexpr int WT_L0 = NF * HID;
// the current layer's W_l as stored, for the data-gradient GEMM (the GEMMs stage their
// weights in 16-byte pieces: every slot starts on a 16-byte boundary)
constexpr int WT_DX = WT_L0 + NLAYER * KC * HID;
constexpr int WT_TOTAL = WT_DX + KC * HID;
static_assert(WT_L0 % 8 == 0 && (KC * HID) % 8 == 0 && WT_DX % 8 == 0, "16-byte aligned BF16 weight slots");

template <int KI, int K1, int NO, int EPI>
int launch_gemm(fe_gnn_s *g, int64_t n, const float *X1, const float *X2, const __nv_bfloat16 *Wt,
                const float *bias, const float *gterm, const float *hres, float *Z, float *Y) {
    const auto kern = k_gemm<KI, K1, NO, EPI>;
    FE_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kTcSmem));
    const int grid = (int)std::max<int64_t>(1, std::min<int64_t>((n + kTcRows - 1) / kTcRows, 152 * 4));
    kern<<<grid, kTcThreads, kTcSmem, g->stream>>>(n, X1, X2, Wt, bias, gterm, hres, Z, Y, g->tc_err.p);
    FE_LAUNCH_CHECK();
    return FE_OK;
}

template <int KI, int K1, int NO>
int launch_wgrad(fe_gnn_s *g, int64_t n, const float *X1, const float *X2, const float *dZ, float *dW) {
    const auto kern = k_gemm_wgrad<KI, K1, NO>;
    FE_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kTcSmem));
    const int grid = (int)std::max<int64_t>(1, std::min<int64_t>((n + kTcRows - 1) / kTcRows, 152 * 4));
    kern<<<grid, kTcThreads, kTcSmem, g->stream>>>(n, X1, X2, dZ, dW, g->tc_err.p);
    FE_LAUNCH_CHECK();
    return FE_OK;
}

// the tensor-core GEMMs' error word, read once the stream has been synchronised
int check_tc(fe_gnn_s *g) {
    int e = 0;
    FE_CUDA(cudaMemcpy(&e, g->tc_err.p, sizeof(int), cudaMemcpyDeviceToHost));
    if (e) {
        set_error("warm-start network: a tensor-core GEMM's MMAs did not complete");
        return FE_CUDA_ERR;
    }
    return FE_OK;
}

int gnn_alloc(fe_gnn_s *g, int64_t n) {
    // whole 32-row SELL slices: spmv64 reads the padding rows of the last slice
    n = (n + 31) / 32 * 32;
    if (n <= g->n_cap) return FE_OK;
    size_t N = (size_t)n;
    FE_CHECK(dalloc(g->F, N * NF));
    FE_CHECK(dalloc(g->Z0, N * HID));
    FE_CHECK(dalloc(g->H, N * HID * (NLAYER + 1)));
    FE_CHECK(dalloc(g->Z, N * HID * NLAYER));
    FE_CHECK(dalloc(g->M, N * HID * NLAYER));
    FE_CHECK(dalloc(g->dH, N * HID));
    FE_CHECK(dalloc(g->dHn, N * HID));
    FE_CHECK(dalloc(g->dX, N * KC));
    FE_CHECK(dalloc(g->dZ, N * HID));
    FE_CHECK(dalloc(g->dM, N * HID));
    FE_CHECK(dalloc(g->inv_deg, N));
    FE_CHECK(dalloc(g->du, N * 2));
    FE_CHECK(dalloc(g->us0, N * 2));
    FE_CHECK(dalloc(g->us1, N * 2));
    FE_CHECK(dalloc(g->gext, N * 2));
    FE_CHECK(dalloc(g->Ag, N * 2));
    FE_CHECK(dalloc(g->bt, N * 2));
    FE_CHECK(dalloc(g->u, N * 2));
    FE_CHECK(dalloc(g->Au, N * 2));
    FE_CHECK(dalloc(g->x0, N * 2));
    g->n_cap = n;
    return FE_OK;
}

int refresh_bf16(fe_gnn_s *g) {
    k_to_bf16_t<<<4, 256, 0, g->stream>>>(g->params.p + P_W0, NF, HID, g->wt.p + WT_W0);
    for (int l = 0; l < NLAYER; ++l)
        k_to_bf16_t<<<16, 256, 0, g->stream>>>(g->params.p + P_L0 + l * L_STRIDE + L_W, KC, HID,
                                               g->wt.p + WT_L0 + l * KC * HID);
    FE_LAUNCH_CHECK();
    return FE_OK;
}

// Problem-dependent inputs: g_ext, b~, node features, inverse degrees.
int prepare(fe_gnn_s *g, fe_handle_s *h, cudaStream_t stream = nullptr) {
    if (h->kind != FE_KIND_ELASTIC_TRI) {
        set_error("the warm-start network is defined for elasticity meshes");
        return FE_BAD_INPUT;
    }
    if (!h->sys_ready) {
        set_error("the warm-start network needs an assembled system");
        return FE_NOT_READY;
    }
    const int64_t n = h->n_nodes, nd = h->n_dof;
    cudaStream_t s = stream ? stream : h->stream;
    g->stream = s;
    FE_CHECK(gnn_alloc(g, n));
    FE_CUDA(cudaMemsetAsync(g->gext.p, 0, nd * sizeof(double), s));
    if (h->n_bc > 0) k_gext<<<g1(h->n_bc), kT, 0, s>>>(h->n_bc, h->bc_dof.p, h->bc_val.p, g->gext.p);
    FE_CHECK(spmv64_on(h, g->gext.p, g->Ag.p, s));
    k_btilde<<<g1(nd), kT, 0, s>>>(nd, h->b.p, g->Ag.p, h->bc_of_dof.p, g->bt.p);
    FE_CHECK(dalloc(g->stats, 8));
    FE_CHECK(dalloc(g->gsum, 8));
    k_init_stats<<<1, 32, 0, s>>>(g->stats.p);
    FE_CUDA(cudaMemsetAsync(g->gsum.p, 0, 8 * sizeof(double), s));
    k_bbox<<<g1(n), kT, 0, s>>>(n, h->coords.p, g->stats.p);
    k_load_moments<<<g1(n), kT, 0, s>>>(n, h->coords.p, g->bt.p, g->stats.p, g->gsum.p);
    k_material_means<<<g1(h->n_elem), kT, 0, s>>>(h->n_elem, h->E.p, h->nu.p, g->gsum.p);
    k_features<<<g1(n), kT, 0, s>>>(n, h->n_elem, h->coords.p, h->bc_of_dof.p, g->stats.p, g->gsum.p, g->F.p);
    k_inv_deg<<<g1(n), kT, 0, s>>>(n, h->blk_ptr.p, h->blk_col.p, g->inv_deg.p);
    FE_LAUNCH_CHECK();
    h->launches += 8 + (h->n_bc > 0 ? 1 : 0);
    return FE_OK;
}

inline float *Hl(fe_gnn_s *g, int l) { return g->H.p + (size_t)l * g->n_cap * HID; }
inline float *Zl(fe_gnn_s *g, int l) { return g->Z.p + (size_t)l * g->n_cap * HID; }
inline float *Ml(fe_gnn_s *g, int l) { return g->M.p + (size_t)l * g->n_cap * HID; }

// async: leave the two sums u.b~, u.A u in acc on the device (no read to the host)
int forward(fe_gnn_s *g, fe_handle_s *h, bool async = false) {
    const int64_t n = h->n_nodes;
    cudaStream_t s = g->stream;
    const float *P = g->params.p;
    FE_CHECK(launch_gemm<NF, NF, HID, EPI_RELU_BIAS>(g, n, g->F.p, nullptr, g->wt.p + WT_W0, P + P_B0, nullptr,
                                                     nullptr, g->Z0.p, Hl(g, 0)));
    FE_CHECK(dalloc(g->colsum, (size_t)(NLAYER + 1) * HID));
    FE_CHECK(dalloc(g->gterm, (size_t)NLAYER * HID));
    FE_CUDA(cudaMemsetAsync(g->colsum.p, 0, (NLAYER + 1) * HID * sizeof(float), s));
    for (int l = 0; l < NLAYER; ++l) {
        const float *LP = P + P_L0 + l * L_STRIDE;
        k_aggregate<false><<<g1(n * 32), kT, 0, s>>>(n, h->blk_ptr.p, h->blk_col.p, g->inv_deg.p, Hl(g, l), Ml(g, l));
        k_colsum<<<std::min<int64_t>((n + 3) / 4, 152 * 4), kT, 0, s>>>(n, Hl(g, l), g->colsum.p + l * HID);
        k_gterm<<<1, HID, 0, s>>>(g->colsum.p + l * HID, 1.f / (float)n, LP + L_U, g->gterm.p + l * HID);
        FE_CHECK(launch_gemm<KC, HID, HID, EPI_LAYER>(g, n, Hl(g, l), Ml(g, l), g->wt.p + WT_L0 + l * KC * HID,
                                                      LP + L_B, g->gterm.p + l * HID, Hl(g, l), Zl(g, l),
                                                      Hl(g, l + 1)));
    }
    k_decode<<<g1(n * 32), kT, 0, s>>>(n, Hl(g, NLAYER), P + P_WD, P + P_BD, h->bc_of_dof.p, g->us0.p);
    float *cur = g->us0.p, *nxt = g->us1.p;
    for (int k = 0; k < NSMOOTH; ++k) {
        k_smooth<false><<<g1(n), kT, 0, s>>>(n, h->blk_ptr.p, h->blk_col.p, g->inv_deg.p, h->bc_of_dof.p, cur, nxt);
        std::swap(cur, nxt);
    }
    k_f32_to_f64<<<g1(2 * n), kT, 0, s>>>(2 * n, cur, g->u.p);
    FE_LAUNCH_CHECK();
    h->launches += 4 + NLAYER * 4 + NSMOOTH;
    // A u_hat and the two dot products u.b~, u.A u
    FE_CHECK(spmv64_on(h, g->u.p, g->Au.p, s));
    FE_CHECK(dalloc(g->acc, 4));
    FE_CUDA(cudaMemsetAsync(g->acc.p, 0, 4 * sizeof(double), s));
    k_dots2<<<g1(h->n_dof), kT, 0, s>>>(h->n_dof, g->u.p, g->bt.p, g->Au.p, g->acc.p);
    FE_LAUNCH_CHECK();
    h->launches += 1;
    if (async) return FE_OK;
    if (!g->acc_host) FE_CUDA(cudaMallocHost((void **)&g->acc_host, 4 * sizeof(double)));
    FE_CUDA(cudaMemcpyAsync(g->acc_host, g->acc.p, 2 * sizeof(double), cudaMemcpyDeviceToHost, s));
    FE_CUDA(cudaStreamSynchronize(s));
    FE_CHECK(check_tc(g));
    g->last_num = g->acc_host[0];
    g->last_den = g->acc_host[1];
    g->last_scale = g->last_den > 0 ? g->last_num / g->last_den : 0.0;
    return FE_OK;
}

// fit = false: energy loss with target energy `energy`; fit = true: mean-squared
// error against the handle's current solution, normalised by its RMS.
int backward(fe_gnn_s *g, fe_handle_s *h, double energy, bool fit, double *loss) {
    const int64_t n = h->n_nodes, nd = h->n_dof;
    cudaStream_t s = g->stream;
    const float *P = g->params.p;
    float *G = g->grad.p;
    FE_CUDA(cudaMemsetAsync(G, 0, P_TOTAL * sizeof(float), s));
    if (fit) {
        FE_CUDA(cudaMemsetAsync(g->acc.p, 0, 4 * sizeof(double), s));
        k_fit_stats<<<g1(nd), kT, 0, s>>>(nd, h->w.x.p, g->gext.p, h->bc_of_dof.p, g->acc.p);
        FE_CUDA(cudaMemcpyAsync(g->acc_host, g->acc.p, 2 * sizeof(double), cudaMemcpyDeviceToHost, s));
        FE_CUDA(cudaStreamSynchronize(s));
        const double ss = g->acc_host[0], nf = g->acc_host[1];
        if (!(ss > 0) || !(nf > 0)) {
            set_error("warm-start fit: the solution has no free displacement");
            return FE_BREAKDOWN;
        }
        const double sigma = sqrt(ss / nf);
        k_fit_grad<<<g1(nd), kT, 0, s>>>(nd, g->u.p, h->w.x.p, g->gext.p, h->bc_of_dof.p, 1.0 / sigma, 1.0 / nf,
                                         g->us0.p, g->acc.p + 2);
        FE_CUDA(cudaMemcpyAsync(g->acc_host + 2, g->acc.p + 2, sizeof(double), cudaMemcpyDeviceToHost, s));
        FE_CUDA(cudaStreamSynchronize(s));
        *loss = g->acc_host[2] / nf;
        h->launches += 2;
    } else {
        const double a = g->last_num, c = g->last_den;
        if (!(c > 0) || !(energy > 0)) {
            set_error("warm-start loss undefined: u_hat . A u_hat or the target energy is not positive");
            return FE_BREAKDOWN;
        }
        *loss = 1.0 - a * a / (c * energy);
        // dL/du = -2a/(c e) b~ + 2a^2/(c^2 e) A u
        const double ca = -2.0 * a / (c * energy), cb = 2.0 * a * a / (c * c * energy);
        k_loss_grad_u<<<g1(nd), kT, 0, s>>>(nd, g->bt.p, g->Au.p, h->bc_of_dof.p, ca, cb, g->us0.p);
        h->launches += 1;
    }
    // adjoint of u = (P S)^K P u_dec:  g <- S^T P g, K times, then P
    float *cur = g->us0.p, *nxt = g->us1.p;
    for (int k = 0; k < NSMOOTH; ++k) {
        k_smooth<true><<<g1(n), kT, 0, s>>>(n, h->blk_ptr.p, h->blk_col.p, g->inv_deg.p, h->bc_of_dof.p, cur, nxt);
        std::swap(cur, nxt);
    }
    k_mask2<<<g1(nd), kT, 0, s>>>(nd, h->bc_of_dof.p, cur);
    k_decode_back<<<g1(n * 32), kT, 0, s>>>(n, Hl(g, NLAYER), P + P_WD, cur, g->dHn.p, G + P_WD, G + P_BD);
    FE_CHECK(dalloc(g->dgb, HID * 2));
    for (int l = NLAYER - 1; l >= 0; --l) {
        const float *LP = P + P_L0 + l * L_STRIDE;
        float *LG = G + P_L0 + l * L_STRIDE;
        // dZ = dH_{l+1} (.) [z_l > 0]
        k_relu_grad<<<g1(n * HID), kT, 0, s>>>(n * HID, g->dHn.p, Zl(g, l), g->dZ.p);
        // dX = dZ W_l^T: the GEMM takes its right operand transposed, [out][in], and
        // (W_l^T)^T = W_l in its stored [128][64] layout, so copy W_l to BF16 as it is
        __nv_bfloat16 *wl = g->wt.p + WT_DX;
        k_to_bf16<<<16, 256, 0, s>>>(LP + L_W, KC * HID, wl);
        FE_CHECK(launch_gemm<HID, HID, KC, EPI_PLAIN>(g, n, g->dZ.p, nullptr, wl, nullptr, nullptr, nullptr,
                                                      nullptr, g->dX.p));
        // weight gradients
        FE_CHECK(launch_wgrad<KC, HID, HID>(g, n, Hl(g, l), Ml(g, l), g->dZ.p, LG + L_W));
        FE_CUDA(cudaMemsetAsync(g->dgb.p + HID, 0, HID * sizeof(float), s));
        k_colsum<<<std::min<int64_t>((n + 3) / 4, 152 * 4), kT, 0, s>>>(n, g->dZ.p, g->dgb.p + HID);
        k_gterm_back<<<1, HID, 0, s>>>(g->colsum.p + l * HID, 1.f / (float)n, LP + L_U, g->dgb.p + HID, LG + L_U,
                                       g->dgb.p);
        // bias gradient = colsum(dZ)
        FE_CUDA(cudaMemcpyAsync(LG + L_B, g->dgb.p + HID, HID * sizeof(float), cudaMemcpyDeviceToDevice, s));
        // dH_l = dH_{l+1} + dX[:, :64] + dg / N ;  dM = dX[:, 64:] ; dH_l += agg^T dM
        k_layer_back_dh<<<g1(n * HID), kT, 0, s>>>(n, g->dHn.p, g->dX.p, g->dgb.p, g->dH.p);
        k_split_dm<<<g1(n * HID), kT, 0, s>>>(n, g->dX.p, g->dM.p);
        k_aggregate<true><<<g1(n * 32), kT, 0, s>>>(n, h->blk_ptr.p, h->blk_col.p, g->inv_deg.p, g->dM.p, g->dH.p);
        std::swap(g->dH.p, g->dHn.p);
        FE_LAUNCH_CHECK();
    }
    // encoder: dZ0 = dH_0 (.) [z0 > 0];  dW0 = F^T dZ0;  db0 = colsum(dZ0)
    k_relu_grad<<<g1(n * HID), kT, 0, s>>>(n * HID, g->dHn.p, g->Z0.p, g->dZ.p);
    FE_CHECK(launch_wgrad<NF, NF, HID>(g, n, g->F.p, nullptr, g->dZ.p, G + P_W0));
    k_colsum<<<std::min<int64_t>((n + 3) / 4, 152 * 4), kT, 0, s>>>(n, g->dZ.p, G + P_B0);
    FE_LAUNCH_CHECK();
    h->launches += 2 + NLAYER * 9 + 3;
    return FE_OK;
}

}  // namespace
}  // namespace fe

using namespace fe;

extern "C" {

int fe_gnn_create(fe_gnn *out) {
    if (!out) {
        set_error("fe_gnn_create: null output");
        return FE_BAD_INPUT;
    }
    fe_gnn_s *g = new fe_gnn_s();
    // BF16 weights: W0 and W_l transposed ([out][in]) for the forward GEMMs, then one
    // slot holding the current layer's W_l as stored, for the data-gradient GEMM
    int st = dalloc(g->params, P_TOTAL);
    if (!st) st = dalloc(g->grad, P_TOTAL);
    if (!st) st = dalloc(g->adam_m, P_TOTAL);
    if (!st) st = dalloc(g->adam_v, P_TOTAL);
    if (!st) st = dalloc(g->wt, (size_t)WT_TOTAL);
    if (!st) st = dalloc(g->tc_err, 1);
    if (st) {
        fe_gnn_destroy(g);
        return st;
    }
    cudaMemset(g->params.p, 0, P_TOTAL * sizeof(float));
    cudaMemset(g->adam_m.p, 0, P_TOTAL * sizeof(float));
    cudaMemset(g->adam_v.p, 0, P_TOTAL * sizeof(float));
    cudaMemset(g->tc_err.p, 0, sizeof(int));
    *out = g;
    return FE_OK;
}

int fe_gnn_destroy(fe_gnn g) {
    if (!g) return FE_OK;
    cudaDeviceSynchronize();
    if (g->ready) cudaEventDestroy(g->ready);
    if (g->assembled) cudaEventDestroy(g->assembled);
    if (g->own) cudaStreamDestroy(g->own);
    dfree(g->params), dfree(g->grad), dfree(g->adam_m), dfree(g->adam_v), dfree(g->wt), dfree(g->tc_err);
    dfree(g->F), dfree(g->Z0), dfree(g->H), dfree(g->Z), dfree(g->M), dfree(g->dH), dfree(g->dHn), dfree(g->dX);
    dfree(g->dZ), dfree(g->dM), dfree(g->inv_deg), dfree(g->colsum), dfree(g->gterm), dfree(g->stats);
    dfree(g->du), dfree(g->dgb), dfree(g->gext), dfree(g->Ag), dfree(g->bt), dfree(g->u), dfree(g->Au);
    dfree(g->x0), dfree(g->acc), dfree(g->us0), dfree(g->us1), dfree(g->gsum);
    if (g->acc_host) cudaFreeHost(g->acc_host);
    delete g;
    return FE_OK;
}

int fe_gnn_num_params(int64_t *n) {
    if (n) *n = P_TOTAL;
    return FE_OK;
}

int fe_gnn_set_params(fe_gnn g, const float *host, int64_t n) {
    if (!g || !host || n != P_TOTAL) {
        set_error("fe_gnn_set_params: expected " + std::to_string(P_TOTAL) + " parameters");
        return FE_BAD_INPUT;
    }
    FE_CUDA(cudaMemcpy(g->params.p, host, n * sizeof(float), cudaMemcpyHostToDevice));
    FE_CUDA(cudaMemset(g->adam_m.p, 0, P_TOTAL * sizeof(float)));
    FE_CUDA(cudaMemset(g->adam_v.p, 0, P_TOTAL * sizeof(float)));
    g->steps = 0;
    return FE_OK;
}

int fe_gnn_get_params(fe_gnn g, float *host, int64_t n) {
    if (!g || !host || n != P_TOTAL) {
        set_error("fe_gnn_get_params: expected " + std::to_string(P_TOTAL) + " parameters");
        return FE_BAD_INPUT;
    }
    FE_CUDA(cudaDeviceSynchronize());
    FE_CUDA(cudaMemcpy(host, g->params.p, n * sizeof(float), cudaMemcpyDeviceToHost));
    return FE_OK;
}

int fe_gnn_features(fe_gnn g, fe_handle h, float *host) {
    if (!g || !h || !host) {
        set_error("fe_gnn_features: null argument");
        return FE_BAD_INPUT;
    }
    FE_CHECK(prepare(g, h));
    FE_CUDA(cudaMemcpyAsync(host, g->F.p, h->n_nodes * NF * sizeof(float), cudaMemcpyDeviceToHost, h->stream));
    FE_CUDA(cudaStreamSynchronize(h->stream));
    g->stream = nullptr;
    return FE_OK;
}

int fe_gnn_predict(fe_gnn g, fe_handle h, double *x0_host, const double **x0_dev, double *scale) {
    if (!g || !h) {
        set_error("fe_gnn_predict: null argument");
        return FE_BAD_INPUT;
    }
    FE_CHECK(prepare(g, h));
    g->stream = h->stream;
    FE_CHECK(refresh_bf16(g));
    FE_CHECK(forward(g, h));
    k_warm_start<<<g1(h->n_dof), kT, 0, h->stream>>>(h->n_dof, g->gext.p, g->u.p, g->last_scale, g->x0.p);
    FE_LAUNCH_CHECK();
    h->launches += 1;
    if (x0_host) {
        FE_CUDA(cudaMemcpyAsync(x0_host, g->x0.p, h->n_dof * sizeof(double), cudaMemcpyDeviceToHost, h->stream));
        FE_CUDA(cudaStreamSynchronize(h->stream));
    }
    FE_CUDA(cudaStreamSynchronize(h->stream));
    g->stream = nullptr;
    if (x0_dev) *x0_dev = g->x0.p;
    if (scale) *scale = g->last_scale;
    return FE_OK;
}

int fe_gnn_predict_async(fe_gnn g, fe_handle h, const double **x0_dev) {
    if (!g || !h || !x0_dev) {
        set_error("fe_gnn_predict_async: null argument");
        return FE_BAD_INPUT;
    }
    if (!g->own) {
        // the lowest priority: blocks of the handle's solve (the multigrid setup's short
        // kernels) are scheduled before the prediction's
        int lo = 0, hi = 0;
        FE_CUDA(cudaDeviceGetStreamPriorityRange(&lo, &hi));
        FE_CUDA(cudaStreamCreateWithPriority(&g->own, cudaStreamNonBlocking, lo));
        FE_CUDA(cudaEventCreateWithFlags(&g->assembled, cudaEventDisableTiming));
        FE_CUDA(cudaEventCreateWithFlags(&g->ready, cudaEventDisableTiming));
    }
    // after the handle's work so far (the assembly), on the network's stream
    FE_CUDA(cudaEventRecord(g->assembled, h->stream));
    FE_CUDA(cudaStreamWaitEvent(g->own, g->assembled, 0));
    FE_CHECK(prepare(g, h, g->own));
    FE_CHECK(refresh_bf16(g));
    FE_CHECK(forward(g, h, true));
    k_warm_start_dev<<<g1(h->n_dof), kT, 0, g->own>>>(h->n_dof, g->gext.p, g->u.p, g->acc.p, g->x0.p);
    FE_LAUNCH_CHECK();
    h->launches += 1;
    FE_CUDA(cudaEventRecord(g->ready, g->own));
    h->x0_ready = g->ready;
    g->stream = nullptr;
    *x0_dev = g->x0.p;
    return FE_OK;
}

int fe_gnn_target_energy(fe_gnn g, fe_handle h, double *energy) {
    if (!g || !h || !energy) {
        set_error("fe_gnn_target_energy: null argument");
        return FE_BAD_INPUT;
    }
    if (!h->have_solution) {
        set_error("fe_gnn_target_energy: solve the problem first");
        return FE_NOT_READY;
    }
    FE_CHECK(prepare(g, h));
    FE_CHECK(dalloc(g->acc, 4));
    FE_CUDA(cudaMemsetAsync(g->acc.p + 2, 0, sizeof(double), h->stream));
    k_energy<<<g1(h->n_dof), kT, 0, h->stream>>>(h->n_dof, g->bt.p, h->w.x.p, g->gext.p, g->acc.p + 2);
    FE_LAUNCH_CHECK();
    h->launches += 1;
    FE_CUDA(cudaMemcpyAsync(energy, g->acc.p + 2, sizeof(double), cudaMemcpyDeviceToHost, h->stream));
    FE_CUDA(cudaStreamSynchronize(h->stream));
    g->stream = nullptr;
    return FE_OK;
}

int fe_gnn_loss_grad(fe_gnn g, fe_handle h, double energy, double *loss, float *grad_host) {
    if (!g || !h || !loss) {
        set_error("fe_gnn_loss_grad: null argument");
        return FE_BAD_INPUT;
    }
    FE_CHECK(prepare(g, h));
    FE_CHECK(refresh_bf16(g));
    FE_CHECK(forward(g, h));
    double l = 0;
    FE_CHECK(backward(g, h, energy, false, &l));
    *loss = l;
    if (grad_host)
        FE_CUDA(cudaMemcpyAsync(grad_host, g->grad.p, P_TOTAL * sizeof(float), cudaMemcpyDeviceToHost, h->stream));
    // the gradient is complete before fe_gnn_adam_step (default stream) may read it
    FE_CUDA(cudaStreamSynchronize(h->stream));
    g->stream = nullptr;
    return FE_OK;
}

int fe_gnn_fit_grad(fe_gnn g, fe_handle h, double *loss, float *grad_host) {
    if (!g || !h || !loss) {
        set_error("fe_gnn_fit_grad: null argument");
        return FE_BAD_INPUT;
    }
    if (!h->have_solution) {
        set_error("fe_gnn_fit_grad: solve the problem first");
        return FE_NOT_READY;
    }
    FE_CHECK(prepare(g, h));
    FE_CHECK(refresh_bf16(g));
    FE_CHECK(forward(g, h));
    double l = 0;
    FE_CHECK(backward(g, h, 0.0, true, &l));
    *loss = l;
    if (grad_host)
        FE_CUDA(cudaMemcpyAsync(grad_host, g->grad.p, P_TOTAL * sizeof(float), cudaMemcpyDeviceToHost, h->stream));
    // the gradient is complete before fe_gnn_adam_step (default stream) may read it
    FE_CUDA(cudaStreamSynchronize(h->stream));
    g->stream = nullptr;
    return FE_OK;
}

int fe_gnn_adam_step(fe_gnn g, float lr, float beta1, float beta2, float eps) {
    if (!g) {
        set_error("fe_gnn_adam_step: null network");
        return FE_BAD_INPUT;
    }
    g->steps += 1;
    float c1 = 1.f - powf(beta1, (float)g->steps), c2 = 1.f - powf(beta2, (float)g->steps);
    // the gradient call synchronised its handle's stream; run on the default stream and
    // finish before any later call reads the parameters on another stream
    k_adam<<<64, 256, 0, 0>>>(P_TOTAL, g->params.p, g->grad.p, g->adam_m.p, g->adam_v.p, lr, beta1, beta2, eps, c1,
                              c2);
    FE_LAUNCH_CHECK();
    FE_CUDA(cudaStreamSynchronize(0));
    return FE_OK;
}

}  // extern "C"
