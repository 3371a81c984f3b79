// Learned surrogate of the particle step (include/sdem_surrogate.h), sm_103a.
//
// Kernels:
//   k_cells / k_edges<count|fill>   cell-grid neighbour graph at radius
//                                   1.5 d_max, CSR by receiver, deterministic
//                                   order (neighbour cell, then sphere index);
//   k_node_feat                     node features (velocity frames, spin,
//                                   size, plane distances) as bf16;
//   k_gemm                          one tensor-core GEMM for every layer of
//                                   the network, forward and backward:
//                                   C = A . B^T over operands that may be
//                                   row-gathered, split in column segments
//                                   (concatenated edge/node inputs) and read
//                                   transposed (weight gradients), with a
//                                   fused bias/ReLU/mask/residual epilogue;
//   k_split_reduce, k_colsum*       deterministic reductions (split-K weight
//                                   gradients, bias gradients);
//   k_segsum, k_gather_add          message aggregation and its adjoints;
//   k_mse, k_adam, k_to_bf16,
//   k_advance                       loss, optimiser, casts, one stride.
//
// GEMM tiling: 128 threads (4 warps) per 64x64 output tile, 32-deep slices of
// the reduction staged in padded shared memory (row stride 40 bf16 = 20
// words, so the 8x4 fragment reads of a warp hit 32 distinct banks), each
// warp a 32x32 sub-tile of 2x4 mma.m16n8k16 (bf16 in, fp32 accumulate).
// Every accumulator element is owned by one thread and summed in a fixed
// reduction order, so results are bit-reproducible run to run.
#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>

#include "../../include/sdem_surrogate.h"

namespace {

constexpr int BM = 64, BN = 64, BK = 32, LDS = BK + 8, GT = 128;
constexpr int kColsumBlocks = 160;

__device__ __forceinline__ uint16_t bf16_bits(float x) { return __bfloat16_as_ushort(__float2bfloat16_rn(x)); }

__device__ __forceinline__ bool bf16_positive(uint16_t b) { return (b & 0x8000u) == 0 && (b & 0x7fffu) != 0; }

// ------------------------------------------------------------------ graph

__global__ void k_cells(int n, const double* __restrict__ posR, sdem_sg_grid g, int* __restrict__ cell) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    int c[3];
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        const double q = (posR[4 * (size_t)i + a] - g.lo[a]) / g.cell;
        c[a] = (q >= 0.0) ? (q < (double)g.dim[a] ? (int)q : g.dim[a] - 1) : 0;
    }
    cell[i] = (c[2] * g.dim[1] + c[1]) * g.dim[0] + c[0];
}

template <bool kFill>
__global__ void k_edges(int n, const double* __restrict__ posR, sdem_sg_grid g, const int* __restrict__ cell,
                        const int* __restrict__ cell_start, const int* __restrict__ sorted, int* __restrict__ degree,
                        const int* __restrict__ row_off, int* __restrict__ dst, int* __restrict__ src,
                        uint16_t* __restrict__ efeat) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const double xi = posR[4 * (size_t)i], yi = posR[4 * (size_t)i + 1], zi = posR[4 * (size_t)i + 2];
    const double ri = posR[4 * (size_t)i + 3];
    const int c = cell[i];
    const int cx = c % g.dim[0], cy = (c / g.dim[0]) % g.dim[1], cz = c / (g.dim[0] * g.dim[1]);
    const double rc2 = g.cutoff * g.cutoff;
    int cnt = 0;
    const int base = kFill ? row_off[i] : 0;
    for (int dz = -1; dz <= 1; ++dz) {
        const int z = cz + dz;
        if (z < 0 || z >= g.dim[2]) continue;
        for (int dy = -1; dy <= 1; ++dy) {
            const int y = cy + dy;
            if (y < 0 || y >= g.dim[1]) continue;
            for (int dx = -1; dx <= 1; ++dx) {
                const int x = cx + dx;
                if (x < 0 || x >= g.dim[0]) continue;
                const int cc = (z * g.dim[1] + y) * g.dim[0] + x;
                const int s1 = cell_start[cc + 1];
                for (int s = cell_start[cc]; s < s1; ++s) {
                    const int j = sorted[s];
                    if (j == i) continue;
                    const double ex = posR[4 * (size_t)j] - xi, ey = posR[4 * (size_t)j + 1] - yi,
                                 ez = posR[4 * (size_t)j + 2] - zi;
                    const double d2 = ex * ex + ey * ey + ez * ez;
                    if (!(d2 < rc2)) continue;
                    if (kFill) {
                        const size_t e = (size_t)base + cnt;
                        dst[e] = i;
                        src[e] = j;
                        const double d = sqrt(d2);
                        const double ov = fmax(ri + posR[4 * (size_t)j + 3] - d, 0.0);
                        __align__(16) uint16_t f[8];
                        f[0] = bf16_bits((float)(ex / g.scale));
                        f[1] = bf16_bits((float)(ey / g.scale));
                        f[2] = bf16_bits((float)(ez / g.scale));
                        f[3] = bf16_bits((float)(d / g.scale));
                        f[4] = bf16_bits((float)(100.0 * ov / g.scale));
                        f[5] = f[6] = f[7] = 0;
                        uint4* o = reinterpret_cast<uint4*>(efeat + e * 16);
                        o[0] = *reinterpret_cast<const uint4*>(f);
                        o[1] = make_uint4(0u, 0u, 0u, 0u);
                    }
                    ++cnt;
                }
            }
        }
    }
    if (!kFill) degree[i] = cnt;
}

__global__ void k_node_feat(int n, const double* __restrict__ posR, const double* __restrict__ vel,
                            const double* __restrict__ omega, int nw, const double* __restrict__ planes, double scale,
                            double vscale, double dclip, uint16_t* __restrict__ nf) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    __align__(16) uint16_t f[32];
#pragma unroll
    for (int k = 0; k < 32; ++k) f[k] = 0;
#pragma unroll
    for (int fr = 0; fr < 3; ++fr)
#pragma unroll
        for (int a = 0; a < 3; ++a) f[fr * 3 + a] = bf16_bits((float)(vel[((size_t)fr * n + i) * 3 + a] / vscale));
    const double x = posR[4 * (size_t)i], y = posR[4 * (size_t)i + 1], z = posR[4 * (size_t)i + 2];
    const double r = posR[4 * (size_t)i + 3];
#pragma unroll
    for (int a = 0; a < 3; ++a) f[9 + a] = bf16_bits((float)(omega[3 * (size_t)i + a] * r / vscale));
    f[12] = bf16_bits((float)(2.0 * r / scale));
    for (int w = 0; w < nw && w < 5; ++w) {
        const double dist = planes[4 * w] * x + planes[4 * w + 1] * y + planes[4 * w + 2] * z + planes[4 * w + 3];
        const double q = fmin(fmax(dist / scale, -dclip), dclip);
        f[13 + w] = bf16_bits((float)(q / dclip));
    }
    uint4* o = reinterpret_cast<uint4*>(nf + (size_t)i * 32);
#pragma unroll
    for (int k = 0; k < 4; ++k) o[k] = reinterpret_cast<const uint4*>(f)[k];
}

// ------------------------------------------------------------------- GEMM

struct Operand {
    const uint16_t* ptr[3];
    const int* idx[3];
    int ld[3];
    int c0[3];
    int nseg;
    int trans;
};

// Address of the 8 elements (row, col..col+7) of an operand.  The segment
// fields are picked with selects, not by a runtime array index, so the
// kernel parameters stay in the constant bank (no local-memory copy).
__device__ __forceinline__ const uint4* chunk_addr(const Operand& op, int row, int col) {
    const bool s1 = op.nseg > 1 && col >= op.c0[1];
    const bool s2 = op.nseg > 2 && col >= op.c0[2];
    const uint16_t* p = s2 ? op.ptr[2] : (s1 ? op.ptr[1] : op.ptr[0]);
    const int* ix = s2 ? op.idx[2] : (s1 ? op.idx[1] : op.idx[0]);
    const int ld = s2 ? op.ld[2] : (s1 ? op.ld[1] : op.ld[0]);
    const int c0 = s2 ? op.c0[2] : (s1 ? op.c0[1] : op.c0[0]);
    const size_t r = ix ? (size_t)ix[row] : (size_t)row;
    return reinterpret_cast<const uint4*>(p + r * ld + (col - c0));
}

// Stages the 64 x 32 tile (dim rows d0.., reduction r0..) of an operand into
// S[d][r].  Elements outside [0, ndim) x [r0, rend) are zero.
__device__ __forceinline__ void load_tile(uint16_t (*S)[LDS], const Operand& op, int d0, int ndim, int r0,
                                          int rend) {
    const int tid = threadIdx.x;
#pragma unroll
    for (int q = 0; q < 2; ++q) {
        const int c = tid + q * GT;  // 256 chunks of 8 elements
        uint4 v = make_uint4(0u, 0u, 0u, 0u);
        if (op.trans == 0) {
            const int d = c >> 2, rc = (c & 3) * 8;
            const int gd = d0 + d, gr = r0 + rc;
            if (gd < ndim && gr < rend) v = __ldg(chunk_addr(op, gd, gr));
            *reinterpret_cast<uint4*>(&S[d][rc]) = v;
        } else {
            const int r = c >> 3, dc = (c & 7) * 8;
            const int gr = r0 + r, gd = d0 + dc;
            if (gr < rend && gd < ndim) v = __ldg(chunk_addr(op, gr, gd));
            const uint16_t* e = reinterpret_cast<const uint16_t*>(&v);
#pragma unroll
            for (int k = 0; k < 8; ++k) S[dc + k][r] = e[k];
        }
    }
}

__device__ __forceinline__ uint32_t lds32(const uint16_t* p) { return *reinterpret_cast<const uint32_t*>(p); }

__device__ __forceinline__ void mma_bf16(float (&d)[4], const uint32_t (&a)[4], const uint32_t (&b)[2]) {
    asm volatile(
        "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
        "{%0,%1,%2,%3};\n"
        : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
        : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b[0]), "r"(b[1]));
}

__global__ void __launch_bounds__(GT) k_gemm(int I, int J, int R, Operand A, Operand B, sdem_sg_epilogue ep,
                                             int rchunk, float* __restrict__ partial) {
    __shared__ __align__(16) uint16_t As[BM][LDS];
    __shared__ __align__(16) uint16_t Bs[BN][LDS];
    const int i0 = blockIdx.x * BM, j0 = blockIdx.y * BN;
    const int rb = blockIdx.z * rchunk;
    const int re = min(R, rb + rchunk);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int g = lane >> 2, t = lane & 3;
    const int wm = (warp & 1) * 32, wn = (warp >> 1) * 32;
    float acc[2][4][4];
#pragma unroll
    for (int a = 0; a < 2; ++a)
#pragma unroll
        for (int b = 0; b < 4; ++b)
#pragma unroll
            for (int c = 0; c < 4; ++c) acc[a][b][c] = 0.f;

    for (int r0 = rb; r0 < re; r0 += BK) {
        load_tile(As, A, i0, I, r0, re);
        load_tile(Bs, B, j0, J, r0, re);
        __syncthreads();
#pragma unroll
        for (int kk = 0; kk < BK; kk += 16) {
            uint32_t af[2][4], bfr[4][2];
#pragma unroll
            for (int mt = 0; mt < 2; ++mt) {
                const int row = wm + mt * 16 + g;
                af[mt][0] = lds32(&As[row][kk + 2 * t]);
                af[mt][1] = lds32(&As[row + 8][kk + 2 * t]);
                af[mt][2] = lds32(&As[row][kk + 2 * t + 8]);
                af[mt][3] = lds32(&As[row + 8][kk + 2 * t + 8]);
            }
#pragma unroll
            for (int nt = 0; nt < 4; ++nt) {
                const int col = wn + nt * 8 + g;
                bfr[nt][0] = lds32(&Bs[col][kk + 2 * t]);
                bfr[nt][1] = lds32(&Bs[col][kk + 2 * t + 8]);
            }
#pragma unroll
            for (int mt = 0; mt < 2; ++mt)
#pragma unroll
                for (int nt = 0; nt < 4; ++nt) mma_bf16(acc[mt][nt], af[mt], bfr[nt]);
        }
        __syncthreads();
    }

#pragma unroll
    for (int mt = 0; mt < 2; ++mt)
#pragma unroll
        for (int nt = 0; nt < 4; ++nt)
#pragma unroll
            for (int h = 0; h < 2; ++h)
#pragma unroll
                for (int q = 0; q < 2; ++q) {
                    const int gi = i0 + wm + mt * 16 + g + h * 8;
                    const int gj = j0 + wn + nt * 8 + 2 * t + q;
                    if (gi >= I || gj >= J) continue;
                    float v = acc[mt][nt][h * 2 + q];
                    if (partial) {
                        partial[((size_t)blockIdx.z * I + gi) * J + gj] = v;
                        continue;
                    }
                    if (ep.bias) v += ep.bias[gj];
                    if (ep.relu) v = fmaxf(v, 0.f);
                    if (ep.mask && !bf16_positive(ep.mask[(size_t)gi * ep.ld_mask + gj])) v = 0.f;
                    if (ep.out) {
                        float* o = ep.out + (size_t)gi * ep.ld_out + gj;
                        *o = ep.accumulate ? *o + v : v;
                    }
                    if (ep.out_bf) ep.out_bf[(size_t)gi * ep.ld_out_bf + gj] = bf16_bits(v);
                    if (ep.resid) {
                        const float w = ep.resid[(size_t)gi * ep.ld_resid + gj] + v;
                        if (ep.res_out) ep.res_out[(size_t)gi * ep.ld_res_out + gj] = w;
                        if (ep.res_out_bf) ep.res_out_bf[(size_t)gi * ep.ld_res_out_bf + gj] = bf16_bits(w);
                    }
                }
}

// ------------------------------------------------------ tcgen05 GEMM
// The same C = A . B^T with the fused epilogue on the 5th-generation tensor
// cores, for the forms without transposed operands or split reductions (the
// forward layers): one CTA of 256 threads per 128 x 128 output tile.
//
// Operand slices (128 rows x 32 reduction elements of A and of B) are
// copied from global memory into shared memory with cp.async -- each 16-byte
// chunk from its own row, so gathered rows and column segments need no
// staging pass -- into the UMMA K-major layout without swizzle: core
// matrices of 8 rows x 16 bytes, (row group, k group) at
// k group * 2048 + row group * 128 bytes, i.e. the descriptor's leading (K)
// byte offset 2048 and stride (M/N) byte offset 128.  Four slice buffers
// form a ring: while the tensor cores work on slice c, the copies of slices
// c+1..c+3 are in flight.  One thread issues tcgen05.mma (kind::f16, bf16 x
// bf16 -> fp32, M = N = 128, K = 16, two per slice) into a 128-column fp32
// accumulator in tensor memory, and tcgen05.commit arrives on the slice
// buffer's mbarrier, which gates the buffer's next copy.  After the last
// slice the accumulator goes through shared memory (tcgen05.ld by lane
// quarter, then whole rows per warp) to a coalesced epilogue.  Every mbarrier wait
// is bounded: on expiry the CTA counts a timeout (sdem_sg_tensor_timeouts)
// and writes zeros.
constexpr int TC_M = 128, TC_N = 128, TC_K = 32, TC_T = 256, TC_STAGES = 4;
constexpr int TC_TILE = TC_M * TC_K * 2;          // bytes of one operand slice (8 KB)
constexpr int TC_SMEM = TC_STAGES * 2 * TC_TILE;  // 64 KB: A and B slices of every stage
constexpr long long TC_WAIT_LIMIT = 1ll << 26;
constexpr uint32_t TC_IDESC = (1u << 4)                        // D: fp32
                              | (1u << 7) | (1u << 10)         // A, B: bf16
                              | ((uint32_t)(TC_N >> 3) << 17)  // N / 8
                              | ((uint32_t)(TC_M >> 4) << 24); // M / 16; both operands K-major
__device__ unsigned int g_tc_timeouts = 0;
int g_tc_enabled = 1;

__device__ __forceinline__ uint32_t smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ uint64_t umma_desc(uint32_t saddr) {
    const uint64_t lbo = 2048, sbo = 128;
    return (uint64_t)((saddr & 0x3FFFFu) >> 4) | ((lbo >> 4) << 16) | ((sbo >> 4) << 32) | (1ull << 46);
}

__device__ __forceinline__ bool mbar_wait(uint32_t bar, uint32_t parity) {
    for (long long it = 0; it < TC_WAIT_LIMIT; ++it) {
        uint32_t done;
        asm volatile(
            "{\n .reg .pred P;\n mbarrier.try_wait.parity.shared::cta.b64 P, [%1], %2;\n selp.u32 %0, 1, 0, P;\n}\n"
            : "=r"(done)
            : "r"(bar), "r"(parity)
            : "memory");
        if (done) return true;
    }
    return false;
}

// cp.async of 16 bytes; src_bytes = 0 fills the chunk with zeros (nothing is read)
__device__ __forceinline__ void cp16(uint32_t dst, const void* src, uint32_t src_bytes) {
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;\n" ::"r"(dst), "l"(src), "r"(src_bytes) : "memory");
}

// rows d0.. (128) x reduction r0..r0+31 of an operand into the core-matrix layout
__device__ __forceinline__ void tc_copy(uint32_t S, const Operand& op, int d0, int ndim, int r0, int rend) {
#pragma unroll
    for (int q = 0; q < 2; ++q) {
        const int c = threadIdx.x + q * TC_T;   // 512 chunks of 8 elements
        const int d = c >> 2, kg = c & 3;
        const int gd = d0 + d, gr = r0 + kg * 8;
        const bool in = gd < ndim && gr < rend;
        const void* src = in ? (const void*)chunk_addr(op, gd, gr) : (const void*)op.ptr[0];
        cp16(S + kg * 2048 + (d >> 3) * 128 + (d & 7) * 16, src, in ? 16u : 0u);
    }
}

__global__ void __launch_bounds__(TC_T, 1) k_gemm_tc(int I, int J, int R, Operand A, Operand B,
                                                      sdem_sg_epilogue ep) {
    extern __shared__ __align__(1024) uint8_t tc_smem[];
    __shared__ __align__(8) uint64_t mbar[TC_STAGES];
    __shared__ uint32_t tmem_slot;
    const uint32_t As0 = smem_u32(tc_smem), Bs0 = As0 + TC_STAGES * TC_TILE;
    const int i0 = blockIdx.x * TC_M, j0 = blockIdx.y * TC_N;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;\n" ::"r"(smem_u32(&tmem_slot)),
                     "r"(TC_N)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;\n" ::: "memory");
    }
    if (threadIdx.x == 0) {
        for (int k = 0; k < TC_STAGES; ++k)
            asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"(smem_u32(&mbar[k])) : "memory");
        asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
    }
    asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
    const uint32_t tmem = tmem_slot;
    const int nch = (R + TC_K - 1) / TC_K;
    bool ok = true;
    // prologue: slices 0 .. STAGES-2 in flight (one commit group each, empty past the end)
#pragma unroll
    for (int k = 0; k < TC_STAGES - 1; ++k) {
        if (k < nch) {
            tc_copy(As0 + k * TC_TILE, A, i0, I, k * TC_K, R);
            tc_copy(Bs0 + k * TC_TILE, B, j0, J, k * TC_K, R);
        }
        asm volatile("cp.async.commit_group;\n" ::: "memory");
    }
    for (int c = 0; c < nch; ++c) {
        const int b = c % TC_STAGES;
        // this thread's copies of slice c have landed; make every thread's
        // visible to the tensor cores
        asm volatile("cp.async.wait_group %0;\n" ::"n"(TC_STAGES - 2) : "memory");
        asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");
        __syncthreads();
        if (threadIdx.x == 0) {
            asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
#pragma unroll
            for (int kk = 0; kk < TC_K / 16; ++kk) {
                const uint64_t ad = umma_desc(As0 + b * TC_TILE + kk * 2 * 2048);
                const uint64_t bd = umma_desc(Bs0 + b * TC_TILE + kk * 2 * 2048);
                const uint32_t acc = (c > 0 || kk > 0) ? 1u : 0u;
                asm volatile(
                    "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
                    " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(tmem),
                    "l"(ad), "l"(bd), "r"(TC_IDESC), "r"(acc)
                    : "memory");
            }
            asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];\n" ::"r"(
                             smem_u32(&mbar[b]))
                         : "memory");
        }
        // slice c + STAGES - 1 goes into the buffer slice c - 1 used: wait
        // for that slice's MMAs first
        const int nx = c + TC_STAGES - 1;
        if (nx < nch) {
            const int bx = nx % TC_STAGES;
            if (c >= 1 && ok) ok = mbar_wait(smem_u32(&mbar[bx]), ((c - 1) / TC_STAGES) & 1);
            tc_copy(As0 + bx * TC_TILE, A, i0, I, nx * TC_K, R);
            tc_copy(Bs0 + bx * TC_TILE, B, j0, J, nx * TC_K, R);
        }
        asm volatile("cp.async.commit_group;\n" ::: "memory");
    }
    asm volatile("cp.async.wait_group 0;\n" ::: "memory");
    if (nch > 0 && ok) ok = mbar_wait(smem_u32(&mbar[(nch - 1) % TC_STAGES]), ((nch - 1) / TC_STAGES) & 1);
    if (!ok && lane == 0) atomicAdd(&g_tc_timeouts, 1u);
    asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
    // Epilogue in two column halves through shared memory (the slice buffers
    // are free now): warp w moves accumulator rows 32 (w mod 4).. and columns
    // 32 (w / 4).. of the half from tensor memory into a padded row-major
    // tile, then every warp writes whole rows, so that the epilogue's global
    // loads and stores are coalesced along j.
    float* T = reinterpret_cast<float*>(tc_smem);   // 128 rows x 65 floats (33 KB)
    const int quarter = warp & 3, sub = warp >> 2;
    const bool valid = nch > 0 && ok;
#pragma unroll 1
    for (int half = 0; half < 2; ++half) {
        const int col = half * 64 + sub * 32;
        uint32_t r[32];
        const uint32_t taddr = tmem + ((uint32_t)(quarter * 32) << 16) + (uint32_t)col;
        asm volatile(
            "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,"
            "%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];\n"
            : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
              "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]),
              "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]),
              "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
            : "r"(taddr));
        asm volatile("tcgen05.wait::ld.sync.aligned;\n" ::: "memory");
        const int row = quarter * 32 + lane;
#pragma unroll
        for (int q = 0; q < 32; ++q) T[row * 65 + sub * 32 + q] = valid ? __uint_as_float(r[q]) : 0.f;
        __syncthreads();
        // 128 rows x 64 columns: warp w writes rows w, w+8, ...; lane l columns l and l+32
#pragma unroll 1
        for (int rr = warp; rr < TC_M; rr += TC_T / 32) {
            const int gi = i0 + rr;
            if (gi >= I) break;
#pragma unroll
            for (int h2 = 0; h2 < 2; ++h2) {
                const int cj = h2 * 32 + lane;
                const int gj = j0 + half * 64 + cj;
                if (gj >= J) continue;
                float v = T[rr * 65 + cj];
                if (ep.bias) v += ep.bias[gj];
                if (ep.relu) v = fmaxf(v, 0.f);
                if (ep.mask && !bf16_positive(ep.mask[(size_t)gi * ep.ld_mask + gj])) v = 0.f;
                if (ep.out) {
                    float* o = ep.out + (size_t)gi * ep.ld_out + gj;
                    *o = ep.accumulate ? *o + v : v;
                }
                if (ep.out_bf) ep.out_bf[(size_t)gi * ep.ld_out_bf + gj] = bf16_bits(v);
                if (ep.resid) {
                    const float w = ep.resid[(size_t)gi * ep.ld_resid + gj] + v;
                    if (ep.res_out) ep.res_out[(size_t)gi * ep.ld_res_out + gj] = w;
                    if (ep.res_out_bf) ep.res_out_bf[(size_t)gi * ep.ld_res_out_bf + gj] = bf16_bits(w);
                }
            }
        }
        __syncthreads();
    }
    asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
    __syncthreads();
    if (warp == 0)
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;\n" ::"r"(tmem), "r"(TC_N) : "memory");
}

__global__ void k_split_reduce(int I, int J, int splits, const float* __restrict__ partial, float* __restrict__ out,
                               int ld_out, int accumulate) {
    const size_t k = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    const size_t IJ = (size_t)I * J;
    if (k >= IJ) return;
    float s = 0.f;
    for (int z = 0; z < splits; ++z) s += partial[z * IJ + k];
    const int i = (int)(k / J), j = (int)(k % J);
    float* o = out + (size_t)i * ld_out + j;
    *o = accumulate ? *o + s : s;
}

// ------------------------------------------------------- reductions, misc

__global__ void k_segsum(int nrows, int J, const int* __restrict__ row_off, const int* __restrict__ perm,
                         const float* __restrict__ x, int ldx, float* __restrict__ out, int ld_out, int accumulate,
                         uint16_t* __restrict__ out_bf, int ld_out_bf) {
    const long long w = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (w >= nrows) return;
    const int row = (int)w;
    const int e0 = row_off[row], e1 = row_off[row + 1];
    for (int j = lane; j < J; j += 32) {
        float s = (accumulate && out) ? out[(size_t)row * ld_out + j] : 0.f;
        for (int e = e0; e < e1; ++e) {
            const size_t sr = perm ? (size_t)perm[e] : (size_t)e;
            s += x[sr * ldx + j];
        }
        if (out) out[(size_t)row * ld_out + j] = s;
        if (out_bf) out_bf[(size_t)row * ld_out_bf + j] = bf16_bits(s);
    }
}

__global__ void k_gather_add(int rows, int J, const int* __restrict__ idx, const float* __restrict__ x, int ldx,
                             const float* __restrict__ y, int ldy, float* __restrict__ out, int ld_out,
                             uint16_t* __restrict__ out_bf, int ld_out_bf) {
    const size_t k = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= (size_t)rows * J) return;
    const size_t e = k / J;
    const int j = (int)(k % J);
    const size_t xr = idx ? (size_t)idx[e] : e;
    float v = x[xr * ldx + j];
    if (y) v = y[e * ldy + j] + v;
    if (out) out[e * ld_out + j] = v;
    if (out_bf) out_bf[e * ld_out_bf + j] = bf16_bits(v);
}

__global__ void k_colsum_part(int M, int J, const float* __restrict__ x, int ldx, float* __restrict__ partial) {
    const int b = blockIdx.x;
    const int chunk = (M + kColsumBlocks - 1) / kColsumBlocks;
    const int r0 = b * chunk, r1 = min(M, r0 + chunk);
    for (int j = threadIdx.x; j < J; j += blockDim.x) {
        float s = 0.f;
        for (int r = r0; r < r1; ++r) s += x[(size_t)r * ldx + j];
        partial[(size_t)b * J + j] = s;
    }
}

__global__ void k_colsum_final(int J, const float* __restrict__ partial, float* __restrict__ out, int accumulate) {
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= J) return;
    float s = 0.f;
    for (int b = 0; b < kColsumBlocks; ++b) s += partial[(size_t)b * J + j];
    out[j] = accumulate ? out[j] + s : s;
}

__global__ void k_mse(int n, int K, const float* __restrict__ pred, int ldp, const float* __restrict__ target,
                      float* __restrict__ rowerr, float* __restrict__ dpred, uint16_t* __restrict__ dpred_bf) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float inv = 2.0f / ((float)n * (float)K);
    float e = 0.f;
    for (int k = 0; k < ldp; ++k) {
        float d = 0.f;
        if (k < K) {
            const float r = pred[(size_t)i * ldp + k] - target[(size_t)i * K + k];
            e += r * r;
            d = r * inv;
        }
        if (dpred) dpred[(size_t)i * ldp + k] = d;
        if (dpred_bf) dpred_bf[(size_t)i * ldp + k] = bf16_bits(d);
    }
    if (rowerr) rowerr[i] = e;
}

__global__ void k_adam(long long n, float* __restrict__ p, const float* __restrict__ g, float* __restrict__ m,
                       float* __restrict__ v, uint16_t* __restrict__ p_bf, float lr, float b1, float b2, float eps,
                       float wd, float c1, float c2) {
    const long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    const float gk = g[k];
    const float mk = b1 * m[k] + (1.f - b1) * gk;
    const float vk = b2 * v[k] + (1.f - b2) * gk * gk;
    m[k] = mk;
    v[k] = vk;
    const float mh = mk / c1, vh = vk / c2;
    const float pk = p[k] - lr * (mh / (sqrtf(vh) + eps) + wd * p[k]);
    p[k] = pk;
    if (p_bf) p_bf[k] = bf16_bits(pk);
}

__global__ void k_to_bf16(long long n, const float* __restrict__ x, uint16_t* __restrict__ y) {
    const long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (k < n) y[k] = bf16_bits(x[k]);
}

__global__ void k_advance(int n, const float* __restrict__ pred, int ldp, double ascale, double gx, double gy,
                          double gz, double h, sdem_sg_box box, double* __restrict__ posR, double* __restrict__ vel,
                          double* __restrict__ omega) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const double g[3] = {gx, gy, gz};
    const double r = posR[4 * (size_t)i + 3];
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        const double acc = ascale * (double)pred[(size_t)i * ldp + a] + g[a];
        const double v0 = vel[(size_t)i * 3 + a];
        double vn = v0 + acc * h;
        double x = posR[4 * (size_t)i + a] + vn * h;
        const double lo = box.lo[a] + r, hi = box.hi[a] - r;
        if (x < lo) {
            x = lo;
            vn = fmax(vn, 0.0);
        } else if (x > hi) {
            x = hi;
            vn = fmin(vn, 0.0);
        }
        vel[((size_t)2 * n + i) * 3 + a] = vel[((size_t)n + i) * 3 + a];
        vel[((size_t)n + i) * 3 + a] = v0;
        vel[(size_t)i * 3 + a] = vn;
        posR[4 * (size_t)i + a] = x;
        const double al = ascale * (double)pred[(size_t)i * ldp + 3 + a] / r;
        omega[(size_t)i * 3 + a] += al * h;
    }
}

// ------------------------------------------------------------------- host

inline cudaStream_t st(void* s) { return reinterpret_cast<cudaStream_t>(s); }

inline int launched() { return cudaGetLastError() == cudaSuccess ? SDEM_SG_OK : SDEM_SG_E_CUDA; }

inline unsigned blocks(long long n, int t) { return (unsigned)((n + t - 1) / t); }

inline bool aligned16(const void* p) { return (reinterpret_cast<uintptr_t>(p) & 15u) == 0; }

// Checks an operand against the dimension its columns cover (total width)
// and converts it to the device form.
bool make_operand(const sdem_sg_operand* in, int cover, Operand* out) {
    if (!in || in->nseg < 1 || in->nseg > 3 || (in->trans != 0 && in->trans != 1)) return false;
    int col = 0;
    for (int s = 0; s < 3; ++s) {
        if (s < in->nseg) {
            if (!in->ptr[s] || !aligned16(in->ptr[s]) || in->width[s] <= 0 || in->width[s] % 8 || in->ld[s] % 8 ||
                in->ld[s] < in->width[s])
                return false;
            out->ptr[s] = in->ptr[s];
            out->idx[s] = in->idx[s];
            out->ld[s] = in->ld[s];
            out->c0[s] = col;
            col += in->width[s];
        } else {
            out->ptr[s] = nullptr;
            out->idx[s] = nullptr;
            out->ld[s] = 0;
            out->c0[s] = 1 << 30;
        }
    }
    out->nseg = in->nseg;
    out->trans = in->trans;
    return col == cover;
}

}  // namespace

extern "C" {

int sdem_sg_cells(int n, const double* posR, const sdem_sg_grid* g, int* cell, void* stream) {
    if (n < 0 || !g || g->cell <= 0.0 || g->dim[0] < 1 || g->dim[1] < 1 || g->dim[2] < 1 ||
        (long long)g->dim[0] * g->dim[1] * g->dim[2] >= (1ll << 31))
        return SDEM_SG_E_ARG;
    if (n == 0) return SDEM_SG_OK;
    if (!posR || !cell) return SDEM_SG_E_ARG;
    k_cells<<<blocks(n, 256), 256, 0, st(stream)>>>(n, posR, *g, cell);
    return launched();
}

int sdem_sg_edge_count(int n, const double* posR, const sdem_sg_grid* g, const int* cell, const int* cell_start,
                       const int* sorted, int* degree, void* stream) {
    if (n < 0 || !g || g->cutoff > g->cell) return SDEM_SG_E_ARG;
    if (n == 0) return SDEM_SG_OK;
    if (!posR || !cell || !cell_start || !sorted || !degree) return SDEM_SG_E_ARG;
    k_edges<false><<<blocks(n, 128), 128, 0, st(stream)>>>(n, posR, *g, cell, cell_start, sorted, degree, nullptr,
                                                           nullptr, nullptr, nullptr);
    return launched();
}

int sdem_sg_edge_fill(int n, const double* posR, const sdem_sg_grid* g, const int* cell, const int* cell_start,
                      const int* sorted, const int* row_off, int* dst, int* src, uint16_t* efeat, void* stream) {
    if (n < 0 || !g || g->cutoff > g->cell || g->scale <= 0.0) return SDEM_SG_E_ARG;
    if (n == 0) return SDEM_SG_OK;
    if (!posR || !cell || !cell_start || !sorted || !row_off || !dst || !src || !efeat || !aligned16(efeat))
        return SDEM_SG_E_ARG;
    k_edges<true><<<blocks(n, 128), 128, 0, st(stream)>>>(n, posR, *g, cell, cell_start, sorted, nullptr, row_off,
                                                          dst, src, efeat);
    return launched();
}

int sdem_sg_node_features(int n, const double* posR, const double* vel, const double* omega, int nw,
                          const double* planes, double scale, double vscale, double dclip, uint16_t* nfeat,
                          void* stream) {
    if (n < 0 || nw < 0 || scale <= 0.0 || vscale <= 0.0 || dclip <= 0.0) return SDEM_SG_E_ARG;
    if (n == 0) return SDEM_SG_OK;
    if (!posR || !vel || !omega || !nfeat || !aligned16(nfeat) || (nw > 0 && !planes)) return SDEM_SG_E_ARG;
    k_node_feat<<<blocks(n, 128), 128, 0, st(stream)>>>(n, posR, vel, omega, nw, planes, scale, vscale, dclip, nfeat);
    return launched();
}

int sdem_sg_gemm(int I, int J, int R, const sdem_sg_operand* a, const sdem_sg_operand* b,
                 const sdem_sg_epilogue* ep, int splits, float* partial, void* stream) {
    if (I < 0 || J < 0 || R < 0 || !ep || splits < 1) return SDEM_SG_E_ARG;
    if (I == 0 || J == 0) return SDEM_SG_OK;
    Operand A, B;
    if (!make_operand(a, a && a->trans ? I : R, &A) || !make_operand(b, b && b->trans ? J : R, &B))
        return SDEM_SG_E_ARG;
    if ((!A.trans || !B.trans) && R % 8) return SDEM_SG_E_ARG;
    if (ep->mask && ep->ld_mask < J) return SDEM_SG_E_ARG;
    if (ep->out && ep->ld_out < J) return SDEM_SG_E_ARG;
    if (ep->out_bf && ep->ld_out_bf < J) return SDEM_SG_E_ARG;
    if (ep->resid && ep->ld_resid < J) return SDEM_SG_E_ARG;
    if ((ep->res_out && ep->ld_res_out < J) || (ep->res_out_bf && ep->ld_res_out_bf < J)) return SDEM_SG_E_ARG;
    long long rchunk = R > 0 ? ((long long)R + splits - 1) / splits : BK;
    rchunk = (rchunk + BK - 1) / BK * BK;
    const int nsplit = R > 0 ? (int)((R + rchunk - 1) / rchunk) : 1;
    const dim3 grid(blocks(I, BM), blocks(J, BN), nsplit);
    if (grid.y > 65535 || grid.z > 65535) return SDEM_SG_E_ARG;
    if (nsplit == 1 && g_tc_enabled && !A.trans && !B.trans) {
        static bool attr = false;
        if (!attr) {
            if (cudaFuncSetAttribute(k_gemm_tc, cudaFuncAttributeMaxDynamicSharedMemorySize, TC_SMEM) != cudaSuccess)
                return SDEM_SG_E_CUDA;
            attr = true;
        }
        const dim3 tgrid(blocks(I, TC_M), blocks(J, TC_N));
        if (tgrid.y > 65535) return SDEM_SG_E_ARG;
        k_gemm_tc<<<tgrid, TC_T, TC_SMEM, st(stream)>>>(I, J, R, A, B, *ep);
        return launched();
    }
    if (nsplit == 1) {
        k_gemm<<<grid, GT, 0, st(stream)>>>(I, J, R, A, B, *ep, (int)rchunk, nullptr);
        return launched();
    }
    if (!partial || !ep->out || ep->bias || ep->relu || ep->mask || ep->out_bf || ep->resid) return SDEM_SG_E_ARG;
    k_gemm<<<grid, GT, 0, st(stream)>>>(I, J, R, A, B, *ep, (int)rchunk, partial);
    if (cudaGetLastError() != cudaSuccess) return SDEM_SG_E_CUDA;
    k_split_reduce<<<blocks((long long)I * J, 256), 256, 0, st(stream)>>>(I, J, nsplit, partial, ep->out, ep->ld_out,
                                                                       ep->accumulate);
    return launched();
}

int sdem_sg_set_tensor_path(int use_tcgen05) {
    if (use_tcgen05 != 0 && use_tcgen05 != 1) return SDEM_SG_E_ARG;
    g_tc_enabled = use_tcgen05;
    return SDEM_SG_OK;
}

int sdem_sg_tensor_timeouts(unsigned int* count) {
    if (!count) return SDEM_SG_E_ARG;
    return cudaMemcpyFromSymbol(count, g_tc_timeouts, sizeof(unsigned int)) == cudaSuccess ? SDEM_SG_OK
                                                                                         : SDEM_SG_E_CUDA;
}

int sdem_sg_segsum(int nrows, int J, const int* row_off, const int* perm, const float* x, int ldx, float* out,
                   int ld_out, int accumulate, uint16_t* out_bf, int ld_out_bf, void* stream) {
    if (nrows < 0 || J < 0 || ldx < J || (out && ld_out < J) || (out_bf && ld_out_bf < J)) return SDEM_SG_E_ARG;
    if (nrows == 0 || J == 0) return SDEM_SG_OK;
    if (!row_off || !x || (!out && !out_bf) || (accumulate && !out)) return SDEM_SG_E_ARG;
    k_segsum<<<blocks((long long)nrows * 32, 256), 256, 0, st(stream)>>>(nrows, J, row_off, perm, x, ldx, out, ld_out,
                                                                        accumulate, out_bf, ld_out_bf);
    return launched();
}

int sdem_sg_gather_add(int rows, int J, const int* idx, const float* x, int ldx, const float* y, int ldy, float* out,
                       int ld_out, uint16_t* out_bf, int ld_out_bf, void* stream) {
    if (rows < 0 || J < 0 || ldx < J || (y && ldy < J) || (out && ld_out < J) || (out_bf && ld_out_bf < J))
        return SDEM_SG_E_ARG;
    if (rows == 0 || J == 0) return SDEM_SG_OK;
    if (!x || (!out && !out_bf)) return SDEM_SG_E_ARG;
    k_gather_add<<<blocks((long long)rows * J, 256), 256, 0, st(stream)>>>(rows, J, idx, x, ldx, y, ldy, out, ld_out,
                                                                          out_bf, ld_out_bf);
    return launched();
}

int sdem_sg_colsum_blocks(void) { return kColsumBlocks; }

int sdem_sg_colsum(int M, int J, const float* x, int ldx, float* out, int accumulate, float* partial, void* stream) {
    if (M < 0 || J < 0 || ldx < J) return SDEM_SG_E_ARG;
    if (J == 0) return SDEM_SG_OK;
    if (!out || !partial || (M > 0 && !x)) return SDEM_SG_E_ARG;
    k_colsum_part<<<kColsumBlocks, 128, 0, st(stream)>>>(M, J, x, ldx, partial);
    if (cudaGetLastError() != cudaSuccess) return SDEM_SG_E_CUDA;
    k_colsum_final<<<blocks(J, 128), 128, 0, st(stream)>>>(J, partial, out, accumulate);
    return launched();
}

int sdem_sg_mse(int n, int K, const float* pred, int ldp, const float* target, float* rowerr, float* dpred,
                uint16_t* dpred_bf, void* stream) {
    if (n < 0 || K < 1 || ldp < K) return SDEM_SG_E_ARG;
    if (n == 0) return SDEM_SG_OK;
    if (!pred || !target) return SDEM_SG_E_ARG;
    k_mse<<<blocks(n, 128), 128, 0, st(stream)>>>(n, K, pred, ldp, target, rowerr, dpred, dpred_bf);
    return launched();
}

int sdem_sg_adam(long long n, float* p, const float* g, float* m, float* v, uint16_t* p_bf, float lr, float beta1,
                 float beta2, float eps, float weight_decay, int step, void* stream) {
    if (n < 0 || step < 1) return SDEM_SG_E_ARG;
    if (n == 0) return SDEM_SG_OK;
    if (!p || !g || !m || !v) return SDEM_SG_E_ARG;
    const float c1 = (float)(1.0 - pow((double)beta1, (double)step));
    const float c2 = (float)(1.0 - pow((double)beta2, (double)step));
    k_adam<<<blocks(n, 256), 256, 0, st(stream)>>>(n, p, g, m, v, p_bf, lr, beta1, beta2, eps, weight_decay, c1, c2);
    return launched();
}

int sdem_sg_to_bf16(long long n, const float* x, uint16_t* y, void* stream) {
    if (n < 0) return SDEM_SG_E_ARG;
    if (n == 0) return SDEM_SG_OK;
    if (!x || !y) return SDEM_SG_E_ARG;
    k_to_bf16<<<blocks(n, 256), 256, 0, st(stream)>>>(n, x, y);
    return launched();
}

int sdem_sg_advance(int n, const float* pred, int ldp, double ascale, double gx, double gy, double gz, double h,
                    const sdem_sg_box* box, double* posR, double* vel, double* omega, void* stream) {
    if (n < 0 || ldp < 6 || !box) return SDEM_SG_E_ARG;
    if (n == 0) return SDEM_SG_OK;
    if (!pred || !posR || !vel || !omega) return SDEM_SG_E_ARG;
    k_advance<<<blocks(n, 128), 128, 0, st(stream)>>>(n, pred, ldp, ascale, gx, gy, gz, h, *box, posR, vel, omega);
    return launched();
}

}  // extern "C"
