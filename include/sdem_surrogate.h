/*
 * sdem_surrogate.h -- C ABI of the learned surrogate of the particle step
 * (libsdem_surrogate.so, sm_103a).
 *
 * The surrogate is a message-passing network over the cell-search neighbour
 * graph (radius 1.5 d_max) that predicts each sphere's mean linear and
 * angular acceleration over a stride of many DEM steps.  It has no
 * counterpart in the reference: it stands beside the plain path
 * (include/sdem_gpu.h), trains on trajectories the plain path generates, and
 * hands control back to the plain path when its error bound is exceeded.
 *
 * Every array argument is a DEVICE pointer (the caller owns the memory);
 * struct arguments (grid, operands, epilogue) are read from host memory at
 * the call.  Each entry point takes a CUDA stream (cudaStream_t passed as
 * void*, NULL = the legacy stream), only enqueues work, and returns 0 or an
 * SDEM_SG_E_* code.  Matrices are
 * row-major; bf16 values travel as uint16_t bit patterns.
 *
 * Network arithmetic: BF16 operands, FP32 accumulation on the tensor cores
 * (mma m16n8k16), FP32 bias/ReLU/residual epilogues, FP32 master weights and
 * Adam state.  Graph construction and features are FP64 (positions) rounded
 * once to FP32 and once to BF16 (round to nearest even).
 */
#ifndef SDEM_SURROGATE_H
#define SDEM_SURROGATE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

enum {
    SDEM_SG_OK = 0,
    SDEM_SG_E_ARG = 1,        /* a size, stride or alignment the kernels do not accept */
    SDEM_SG_E_CUDA = 2,       /* a launch failed (cudaGetLastError) */
};

/* Uniform cell grid of the neighbour search.  cell >= cutoff, so the edges
 * of a sphere are found in its own and the 26 surrounding cells.  Positions
 * outside the grid are clamped into the border cells (a clamped pair within
 * the cutoff still lies in neighbouring cells). */
typedef struct sdem_sg_grid {
    double lo[3];      /* grid origin */
    double cell;       /* cell edge */
    double cutoff;     /* edge radius (1.5 d_max) */
    double scale;      /* feature length scale (d_max) */
    int dim[3];        /* cells per axis */
    int pad_;
} sdem_sg_grid;

/* cell[i] = (iz*dim[1] + iy)*dim[0] + ix of sphere i (posR: n x 4, x y z r). */
int sdem_sg_cells(int n, const double* posR, const sdem_sg_grid* g, int* cell, void* stream);

/* Edge count of each receiver i: spheres j != i with |x_j - x_i|^2 < cutoff^2,
 * found through cell_start (ncell+1 offsets) and sorted (sphere indices
 * ordered by (cell, index)). */
int sdem_sg_edge_count(int n, const double* posR, const sdem_sg_grid* g, const int* cell,
                       const int* cell_start, const int* sorted, int* degree, void* stream);

/* Edges in CSR order: the row of receiver i (row_off[i] .. row_off[i+1]) lists
 * its senders in the order neighbour cell (dz, dy, dx from -1 to 1, dx
 * fastest), then sphere index.  dst[e] = i, src[e] = j; efeat[e] (16 bf16):
 * (x_j - x_i)/scale (3), |x_j - x_i|/scale, 100 max(r_i + r_j - |x_j - x_i|, 0)/scale,
 * zeros. */
int sdem_sg_edge_fill(int n, const double* posR, const sdem_sg_grid* g, const int* cell,
                      const int* cell_start, const int* sorted, const int* row_off, int* dst, int* src,
                      uint16_t* efeat, void* stream);

/* Node features (32 bf16 per sphere): three velocity frames v(t), v(t-S),
 * v(t-2S) divided by vscale (9), omega r / vscale (3), 2r/scale, the signed
 * distances to up to 5 planes (n.x + d, planes: nw x 4 doubles nx ny nz d)
 * divided by scale and clipped to [-dclip, dclip] then divided by dclip (5),
 * zeros.  vel: 3 x n x 3 (frame, sphere, xyz); omega: n x 3. */
int sdem_sg_node_features(int n, const double* posR, const double* vel, const double* omega, int nw,
                          const double* planes, double scale, double vscale, double dclip, uint16_t* nfeat,
                          void* stream);

/* A matrix operand of sdem_sg_gemm: up to three column segments, each an
 * optionally row-gathered bf16 matrix.  Element (row, col) with col in
 * segment s (segments are consecutive, first at column 0) is
 *   ptr[s][(idx[s] ? idx[s][row] : row) * ld[s] + col - col0(s)].
 * Widths and ld are multiples of 8, pointers 16-byte aligned.  trans = 0: the
 * operand's rows run along the output dimension and its columns along the
 * reduction; trans = 1: the other way round. */
typedef struct sdem_sg_operand {
    const uint16_t* ptr[3];
    const int* idx[3];
    int ld[3];
    int width[3];
    int nseg;
    int trans;
} sdem_sg_operand;

/* Epilogue of sdem_sg_gemm, applied to v = sum_r A(i,r) B(j,r) per output
 * element: v += bias[j]; v = max(v, 0) if relu; v = 0 where mask (bf16) is not
 * positive; out = v (or out += v if accumulate), out_bf = bf16(v); and with
 * resid: w = resid + v, res_out = w, res_out_bf = bf16(w).  Any pointer may
 * be NULL.  With splits > 1 only out/accumulate apply. */
typedef struct sdem_sg_epilogue {
    const float* bias;
    int relu;
    int accumulate;
    const uint16_t* mask; int ld_mask;
    float* out; int ld_out;
    uint16_t* out_bf; int ld_out_bf;
    const float* resid; int ld_resid;
    float* res_out; int ld_res_out;
    uint16_t* res_out_bf; int ld_res_out_bf;
} sdem_sg_epilogue;

/* C (I x J) = sum over r < R of A(i, r) B(j, r) on the tensor cores.
 * splits > 1 splits the reduction over blocks; `partial` (splits x I x J
 * floats) holds the per-split sums, added in split order (deterministic). */
int sdem_sg_gemm(int I, int J, int R, const sdem_sg_operand* a, const sdem_sg_operand* b,
                 const sdem_sg_epilogue* ep, int splits, float* partial, void* stream);

/* Which tensor-core kernel sdem_sg_gemm uses for the forms without
 * transposed operands or split reductions: 1 (default) the tcgen05/TMEM
 * kernel, 0 the warp-level mma.sync kernel (kept for the other forms). */
int sdem_sg_set_tensor_path(int use_tcgen05);
/* Number of tcgen05 GEMM blocks whose bounded mbarrier wait expired (0
 * expected; such a block writes zeros instead of its products). */
int sdem_sg_tensor_timeouts(unsigned int* count);

/* out[i] (J floats) = (accumulate ? out[i] : 0) + sum over e in row_off[i] ..
 * row_off[i+1] of x[perm ? perm[e] : e]; out_bf = bf16(out) when given.
 * Rows are summed in list order (deterministic). */
int sdem_sg_segsum(int nrows, int J, const int* row_off, const int* perm, const float* x, int ldx, float* out,
                   int ld_out, int accumulate, uint16_t* out_bf, int ld_out_bf, void* stream);

/* out[e] = (y ? y[e] : 0) + x[idx ? idx[e] : e] (J floats per row);
 * out_bf = bf16(out) when given. */
int sdem_sg_gather_add(int rows, int J, const int* idx, const float* x, int ldx, const float* y, int ldy,
                       float* out, int ld_out, uint16_t* out_bf, int ld_out_bf, void* stream);

/* Column sums of x (M x J, fp32): out[j] (+)= sum_i x[i][j], in a fixed
 * order; partial holds sdem_sg_colsum_blocks() x J floats. */
int sdem_sg_colsum_blocks(void);
int sdem_sg_colsum(int M, int J, const float* x, int ldx, float* out, int accumulate, float* partial,
                   void* stream);

/* Mean-squared error of pred (n x ldp, first K columns) against target
 * (n x K): rowerr[i] = sum_k (pred - target)^2; dpred = 2 (pred - target) /
 * (n K) in the first K columns and 0 in the rest (fp32 and bf16, ld ldp). */
int sdem_sg_mse(int n, int K, const float* pred, int ldp, const float* target, float* rowerr, float* dpred,
                uint16_t* dpred_bf, void* stream);

/* Adam with decoupled weight decay over a flat fp32 parameter vector;
 * p_bf (optional) receives bf16(p) after the update. */
int sdem_sg_adam(long long n, float* p, const float* g, float* m, float* v, uint16_t* p_bf, float lr,
                 float beta1, float beta2, float eps, float weight_decay, int step, void* stream);

/* bf16(x) elementwise (round to nearest even). */
int sdem_sg_to_bf16(long long n, const float* x, uint16_t* y, void* stream);

/* Planes of the box that hold the spheres in a surrogate stride: x_a >= lo[a]
 * + r and x_a <= hi[a] - r (use -/+1e300 for an open side). */
typedef struct sdem_sg_box {
    double lo[3];
    double hi[3];
} sdem_sg_box;

/* One surrogate stride of length h: with a_k = ascale * pred[i][k] + g_k (k <
 * 3, g = (gx, gy, gz)) and alpha_k = ascale * pred[i][3+k] / r_i, v' = v(t) + a h,
 * x' = x + v' h, omega' = omega + alpha h; a sphere that would cross a plane of
 * the box is put back against it and keeps no velocity into it; the velocity
 * frames shift (vel[2] <- vel[1] <- vel[0] <- v').  pred: n x ldp fp32. */
int sdem_sg_advance(int n, const float* pred, int ldp, double ascale, double gx, double gy, double gz, double h,
                    const sdem_sg_box* box, double* posR, double* vel, double* omega, void* stream);

#ifdef __cplusplus
}
#endif

#endif
