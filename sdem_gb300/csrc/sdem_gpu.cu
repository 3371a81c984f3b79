// sdem_gpu.cu -- GB300 (sm_103a) kernels and C ABI for sDEM's per-step
// particle hot path.  Build: nvcc -gencode arch=compute_103a,code=sm_103a
// -O3 -fmad=false (see sdem_gb300/build.py).
//
// One step (the body of DEMS_iterate, Prtcl_DEMSystem.f90:214-247) is:
//   k_step_begin                       UpdateNearPrtclsPW (Prtcl_ContactSearchPW.f90:159-235),
//                                      device-predicated on iter >= Next_iter_update; the
//                                      step's image and gather-order counters reset
//   k_ghost_*                          PC_Comm_For_Cntct on one rank (periodic directions only):
//                                      images of the particles near periodic faces, in the
//                                      reference's pass order, as ordered stream compactions
//   k_bin, scan, k_scatter, k_cellorder
//                                      NBSM_clcBoxIndex + Y/X/Z lists (Prtcl_NBS_Munjiza.f90:163-296)
//                                      as a counting sort; within a cell particles are ordered by
//                                      decreasing index, the order the reference's Z lists walk; the
//                                      binning also makes the single-precision prefilter copy and
//                                      each particle's cell coordinates
//   k_search                           LoopNBSMask + FineSearch2/3 (:302-473, :503-557): one thread per
//                                      target particle, same 13-cell half shell + same-cell tail, same
//                                      exact FP64 overlap test; contacts go to the target's row (in visit
//                                      order) and an entry (target, slot) to the partner's in-list
//   k_wall_detect                      FindContactsPW's detection (:298-319) over the near-wall mask,
//                                      and the contact count of every particle for the gather order
//   scan, k_row_fill                   row offsets (CSR) and each contact's row
//   k_force                            Find_insert history lookup + ContactForce_PP / _PPG
//                                      (Prtcl_CL_and_CF.f90:142-198, 256-296, 732-798): one thread per
//                                      contact, full warps of FP64 work
//   k_wall_force                       ContactForce_PW (:832-856), one thread per wall contact
//   k_degree_scatter                   particles grouped by contact count (the gather order), one
//                                      record per gather position with what the gather reads first
//
// Search, row offsets, row fill and forces run in chunks of target sort
// positions on two streams, so that the search of one chunk (integer and
// memory work) overlaps the force kernel of the one before (FP64 work); wall
// detection, wall forces and the gather order follow the searches on the
// second stream, beside the forces.
//   k_gather                           per particle, sums its contact records in the reference's scatter
//                                      order (a deterministic gather; records signed for the row's
//                                      target, moments scaled by the particle's own radius), then its
//                                      wall contacts in near-list order
//   k_integrate                        clc_Acceleration (Prtcl_DEMSystem.f90:166-181), Prtcl_Integrate
//                                      (Prtcl_Integration.f90:15-88) and the periodic wrap, in index
//                                      order
//   k_finish                           one-rank out-of-domain delete (Prtcl_Comm.f90:1569-1840),
//                                      iterNumber += 1, counters
// RemvReleased/PreIteration have no kernel: the history of step n+1 is exactly
// the contact records written at step n (double-buffered, keyed by particle id).
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <unordered_map>
#include <vector>

#include "../../include/sdem_gpu.h"
#include "dem_device.cuh"
#include "fp64_int.cuh"

using sdem::dbl4;
using sdem::make_dbl4;
using sdem::r3;

namespace {

constexpr int kThreads = 256;
constexpr int kMaxK = 64;         // row / in-list capacity limit (6-bit slot in the in-list key)
constexpr int kKw = 4;            // wall contacts per particle
constexpr int kMaxWalls = 64;     // near-wall mask is 64 bits
constexpr int kOutCap = 4096;     // out-of-domain deletions per step
constexpr int kScanThreads = 256, kScanItems = 32;
constexpr int kScanTile = kScanThreads * kScanItems;   // elements per scan block
constexpr int kDegBuckets = 64;   // gather-order buckets by number of contact records
#ifndef SDEM_PIPELINE_CHUNKS
#define SDEM_PIPELINE_CHUNKS 2
#endif
constexpr int kChunks = SDEM_PIPELINE_CHUNKS;   // search/force pipeline chunks per step (default)
constexpr int kMaxChunks = 4;                   // most chunks sdem_set_launch accepts
constexpr int kSearchBlocksPerSM = 6;           // k_search's register budget: resident blocks of kThreads
constexpr int kForceBlocksPerSM = 3;            // k_force blocks per SM in the pipeline (default)
#ifndef SDEM_FORCE_MIN_BLOCKS
#define SDEM_FORCE_MIN_BLOCKS 3    // k_force blocks of 256 threads per SM its register budget allows
#endif
#ifndef SDEM_SEARCH_PREFETCH
#define SDEM_SEARCH_PREFETCH 0     // 1: k_search requests the next candidate's record before testing one
#endif
constexpr int kMaxLevels = 6;     // hierarchical search levels (Init_Munjiza_Hrchl caps at 6)

// One level of the hierarchical search: a grid of cells 2^(mult-1) times
// finer than the base grid; its cells sit at [base, base + nx*ny*nz) of the
// concatenated cell arrays (the finest level first, the order of the search).
struct LevelGrid {
  int nx, ny, nz, mult;
  long long base;
  double cell;
  float cellf;
  fpi::Divisor div;   // the cell length as a divisor (reciprocal refined once, on the host)
};
constexpr int kImgFlag = 1 << 30; // c_ogid bit: a pair with a periodic image (ids < 2^30)

// Phases of one step, for the optional per-phase timing (sdem_profile_*).
enum Phase { PH_WALL, PH_BIN, PH_SCAN_CELLS, PH_SCATTER, PH_CELLORDER, PH_SEARCH, PH_SCAN_ROWS, PH_ROW_FILL,
             PH_FORCE, PH_WALL_FORCE, PH_GATHER, PH_DELETE, PH_END, kPhases };
const char* const kPhaseNames[kPhases] = {"wall_refresh", "bin", "scan_cells", "scatter", "cellorder", "search",
                                          "scan_rows", "row_fill", "force", "wall_force", "gather_integrate",
                                          "delete", "step_end"};

// What the gather reads first for the sphere at one gather position, written
// by the degree scatter in index order (coalesced there) so that the gather
// reads one record instead of several scattered values.
struct __align__(32) GRec {
  int p;        // the sphere
  int s;        // its sort position
  int own_a;    // its row start
  int counts;   // row length << 16 | in-list length << 8 | wall contacts
  double r;     // its radius
  double pad;
};

// ---------------------------------------------------------------------------
// The force kernel's record of one contact for the gather, 96 bytes in one
// place (the gather reads all three of a contact together).
struct __align__(32) ContactRec {
  dbl4 S;    // Fnij + Ftij, signed for the row's target
  dbl4 M;    // Moment = Norm_v x Ftij (each side's gather scales it by its own radius)
  dbl4 Mr;   // Mrij, signed for the row's target
};

// Device view of one handle, passed by value to every kernel.
struct Dev {
  int ncap, n_launch;
  int* n;  // device particle count (changes on deletion)
  // periodic images: ghosts live at indices [n, n + ng) of the search arrays
  // (gid, ptype, posr, vel0, rv0 and the binning/row arrays, stride nall)
  int nall, nall_launch, gcap;
  // hierarchical search (CS_Method 2): levels, 0 = coarsest
  int hier, nlvl;
  LevelGrid lv[kMaxLevels];
  const int* type_lvl;   // level of each type
  // fixed spheres: appended to the search arrays after the images every step
  int nfix;
  const int *fix_gid, *fix_ptype;
  const dbl4* fix_posr;
  int* ng;
  int* nt;   // n + ng: particles the search sees
  int per[3];
  double3 Lbox;
  double lencs;   // LenForCS = Prtcl_cs_ratio * maxD (Prtcl_Comm.f90:80-81)
  int *gflag, *goff;
  int max_gid, K, Kin, ccap;
  int tsize, rsize, pi, pri, quirk;
  sdem::LawCfg law;
  double3 g;
  double cell, x0, y0, z0;
  int nx, ny, nz;
  long long ncell;
  double3 dmin, dmax;
  // tables
  int nT, nWT;
  const double *radius, *mass, *inertia, *bpp, *bpw;
  int nw;
  const double* walls;
  const int* wflags;
  double dx1, dx2, max_wall_vel;
  int wall_max_update_iter;
  // particle state
  int *gid, *ptype, *usrmark;
  dbl4* posr;
  dbl4 *vel0, *vel1, *vel2, *acc0, *acc1, *acc2;
  dbl4 *theta, *rv0, *rv1, *rv2, *ra0, *ra1, *ra2;
  dbl4 *F, *T;
  unsigned long long* near_mask;
  // binning
  int *cell_of, *cell_cnt, *cell_start, *tmp_rank, *tmp_sorted, *sorted, *sortpos;
  float4* spos;      // cell-sorted single-precision copy (offsets in the cell, r) for the prefilter
  float4* pf;        // the same per particle index, written by the binning
  int4* pcell;   // per index: the cell (ix, iy, iz, key in its level's grid), written by the binning
  fpi::Divisor cdiv; // the cell length as a divisor
  float pf_margin;   // prefilter margin, bounds the single-precision distance error
  float cellf;       // cell size in single precision
  // rows and in-lists
  int *row_cnt, *row_partner, *row_off;
  int* in_cnt;
  unsigned* in_list;
  // contact records
  int *c_ogid, *c_pgid;
  const int* c_pgid_prev;
  dbl4* c_hist;
  const dbl4* c_hist_prev;
  struct ContactRec* c_rec;   // per contact: S = Fnij+Ftij and Mr = Mrij signed for the row's target, M = n x Ftij
  // contact history by the reference's bucket owner (Find_insert's bkt_id):
  // the lower id for particle-particle pairs, the local particle for a pair
  // with a periodic image; own_c lists this step's contacts of each owner id
  int Ko;
  int* c_row;   // row (target sort position) of each contact
  int* own_cnt;
  int2* own_c;   // (contact index, partner id): the lookup reads the partner ids of one owner in one sector
  const int* own_cnt_prev;
  const int2* own_c_prev;
  int *wh_cnt, *wh_wall;
  dbl4* wh_hist;
  // wall contacts of this step: per particle up to kKw slots (decreasing wall
  // index), and a compact list (particle << 3 | slot) for the force kernel
  int* w_cnt;
  int* w_wall;
  dbl4* w_geo;       // (nv, ovrlp)
  dbl4 *w_S, *w_M, *w_Mr;
  int* wl;
  int* wl_cnt;
  // gather order: particles bucketed by their number of contact records, so a
  // warp's summation loops run the same trip count
  int *deg_cnt, *deg_of, *deg_rank;
  struct GRec* gorder;   // per gather position: what the gather reads first
  const int *wh_cnt_prev, *wh_wall_prev;
  const dbl4* wh_hist_prev;
  // status and scalars
  int* status;                    // [0] error code, [1] detail
  unsigned long long* counters;   // [0] candidates, [1] PW contacts, [2..4] sums since upload: PP, PW, steps,
                                  // [5] contacts with periodic images (numCntcts(2))
  unsigned long long* red;        // per block of k_step_begin: max |v| bits, max |a| bits
  int* iter;
  int* next_update;
  int* out_cnt;
  int* ticket;   // last-block ticket of k_step_begin
  int* out_list;
  int* moves;      // [0] count, then (dst, src) pairs
  int* map_pos;    // deletion scratch
  int* map_id;
};

__device__ __forceinline__ void raise(const Dev& d, int code, int detail) {
  if (atomicCAS(d.status, 0, code) == 0) d.status[1] = detail;
}

// ---------------------------------------------------------------------------
// Exclusive scan of int32 (n elements) into out[0..n], out[n] = total, in
// three launches: tile sums, a scan of the tile sums, the tiles.  A tile is
// 256 threads x 32 elements; full, 16-byte-aligned tiles move as int4
// (each load instruction covers 512 contiguous bytes of a warp).
__device__ __forceinline__ bool scan_vec_ok(const int* p, long long base, long long n) {
  return base + kScanTile <= n && ((reinterpret_cast<uintptr_t>(p) & 15u) == 0);
}

__global__ void __launch_bounds__(kScanThreads) k_scan_reduce(const int* __restrict__ in, long long n,
                                                               int* __restrict__ bsum) {
  __shared__ int warp_sums[kScanThreads / 32];
  const long long base = (long long)blockIdx.x * kScanTile;
  int s = 0;
  if (scan_vec_ok(in, base, n)) {
    const int4* v = reinterpret_cast<const int4*>(in + base);
#pragma unroll
    for (int j = 0; j < kScanItems / 4; j++) {
      const int4 q = v[j * kScanThreads + threadIdx.x];
      s += (q.x + q.y) + (q.z + q.w);
    }
  } else {
    for (int e = threadIdx.x; e < kScanTile; e += kScanThreads)
      if (base + e < n) s += in[base + e];
  }
  for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
  if ((threadIdx.x & 31) == 0) warp_sums[threadIdx.x >> 5] = s;
  __syncthreads();
  if (threadIdx.x == 0) {
    int v = 0;
    for (int w = 0; w < kScanThreads / 32; w++) v += warp_sums[w];
    bsum[blockIdx.x] = v;
  }
}

__device__ __forceinline__ int block_exclusive_scan_1024(int v, int* sh, int* total) {
  // inclusive warp scan
  int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  int x = v;
  for (int o = 1; o < 32; o <<= 1) {
    int y = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= o) x += y;
  }
  if (lane == 31) sh[wid] = x;
  __syncthreads();
  if (wid == 0) {
    int w = (lane < (int)(blockDim.x >> 5)) ? sh[lane] : 0;
    int z = w;
    for (int o = 1; o < 32; o <<= 1) {
      int y = __shfl_up_sync(0xffffffffu, z, o);
      if (lane >= o) z += y;
    }
    sh[lane] = z - w;  // exclusive warp offsets
    if (lane == 31) sh[32] = z;
  }
  __syncthreads();
  int r = sh[wid] + x - v;
  *total = sh[32];
  __syncthreads();
  return r;
}

__global__ void k_scan_blocks(int* bsum, int nb) {
  __shared__ int sh[33];
  int carry = 0;
  for (int base = 0; base < nb; base += 1024) {
    int i = base + threadIdx.x;
    int v = (i < nb) ? bsum[i] : 0;
    int tot;
    int e = block_exclusive_scan_1024(v, sh, &tot);
    if (i < nb) bsum[i] = e + carry;
    carry += tot;
  }
}

// out[i] = *offset + sum of in[0..i), out[n] = the total (offset may be null).
// The tile goes through shared memory (padded: element e at e + e/32, so that
// both the striped int4 copies and the per-thread runs of 32 are free of bank
// conflicts); each thread scans its 32 consecutive elements, the block scans
// the 256 thread totals.
__global__ void __launch_bounds__(kScanThreads) k_scan_apply(const int* __restrict__ in, long long n,
                                                              const int* __restrict__ bsum, int* __restrict__ out,
                                                              const int* __restrict__ offset) {
  __shared__ int sh[kScanTile + kScanTile / 32];
  __shared__ int wsum[kScanThreads / 32 + 1];
  const int t = threadIdx.x;
  const long long base = (long long)blockIdx.x * kScanTile;
  auto pad = [](int e) { return e + (e >> 5); };
  if (scan_vec_ok(in, base, n)) {
    const int4* v = reinterpret_cast<const int4*>(in + base);
#pragma unroll
    for (int j = 0; j < kScanItems / 4; j++) {
      const int4 q = v[j * kScanThreads + t];
      const int e = pad((j * kScanThreads + t) * 4);
      sh[e] = q.x;
      sh[e + 1] = q.y;
      sh[e + 2] = q.z;
      sh[e + 3] = q.w;
    }
  } else {
    for (int e = t; e < kScanTile; e += kScanThreads) sh[pad(e)] = base + e < n ? in[base + e] : 0;
  }
  __syncthreads();
  int loc[kScanItems];
  int sum = 0;
#pragma unroll
  for (int i = 0; i < kScanItems; i++) {
    const int v = sh[t * (kScanItems + 1) + i];
    loc[i] = sum;
    sum += v;
  }
  // exclusive scan of the thread totals
  const int lane = t & 31, w = t >> 5;
  int x = sum;
  for (int o = 1; o < 32; o <<= 1) {
    const int y = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= o) x += y;
  }
  if (lane == 31) wsum[w] = x;
  __syncthreads();
  if (t == 0) {
    int acc = 0;
    for (int k = 0; k < kScanThreads / 32; k++) {
      const int c = wsum[k];
      wsum[k] = acc;
      acc += c;
    }
    wsum[kScanThreads / 32] = acc;
  }
  __syncthreads();
  const int carry = bsum[blockIdx.x] + (offset ? *offset : 0);
  const int first = carry + wsum[w] + x - sum;
#pragma unroll
  for (int i = 0; i < kScanItems; i++) sh[t * (kScanItems + 1) + i] = first + loc[i];
  __syncthreads();
  if (scan_vec_ok(out, base, n)) {
    int4* v = reinterpret_cast<int4*>(out + base);
#pragma unroll
    for (int j = 0; j < kScanItems / 4; j++) {
      const int e = pad((j * kScanThreads + t) * 4);
      v[j * kScanThreads + t] = make_int4(sh[e], sh[e + 1], sh[e + 2], sh[e + 3]);
    }
  } else {
    for (int e = t; e < kScanTile; e += kScanThreads)
      if (base + e < n) out[base + e] = sh[pad(e)];
  }
  if (blockIdx.x == gridDim.x - 1 && t == 0) out[n] = carry + wsum[kScanThreads / 32];
}

// ---------------------------------------------------------------------------
// The start of a step.  UpdateNearPrtclsPW (Prtcl_ContactSearchPW.f90:159-235)
// when iter >= Next_iter_update: the near-wall bit mask of every particle
// (walls whose AABB +- DeltaXmax2 holds it) and max |v|, max |a|, reduced per
// block into partials; the last block to finish reduces the partials and
// computes the next refresh iteration.  Every step: the image and
// gather-order counters reset.  A fixed grid (grid-stride over particles), so
// that a step without refresh costs a few hundred block launches.
constexpr int kBeginBlocksPerSM = 4;

__device__ __forceinline__ void reset_step_counters(const Dev& d) {
  *d.ng = 0;
  *d.nt = *d.n;
  for (int b = 0; b < kDegBuckets; b++) d.deg_cnt[b] = 0;   // gather-order buckets of this step
}

__global__ void __launch_bounds__(kThreads) k_step_begin(Dev d) {
  const bool refresh = *d.iter >= *d.next_update;
  if (!refresh) {
    if (blockIdx.x == 0 && threadIdx.x == 0) reset_step_counters(d);
    return;
  }
  // expanded wall boxes, pmin = min - DeltaXmax2 and pmax = max + DeltaXmax2
  // (FP64, as the reference), once per block; the tests run on the integer pipes
  __shared__ double box[64][6];
  for (int e = threadIdx.x; e < d.nw * 6; e += blockDim.x) {
    const int k = e / 6, c = e % 6;
    const double* r = d.walls + k * SDEM_W_SIZE;
    box[k][c] = c < 3 ? r[SDEM_W_MIN + c] - d.dx2 : r[SDEM_W_MAX + c - 3] + d.dx2;
  }
  __syncthreads();
  const int n = *d.n;
  // non-negative doubles order like their bit patterns
  unsigned long long vb = 0ull, ab = 0ull;
  for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < n; p += gridDim.x * blockDim.x) {
    const dbl4 P = d.posr[p];
    unsigned long long mask = 0ull;
    for (int k = 0; k < d.nw; k++) {
      if (fpi::ge(P.x, box[k][0]) && fpi::le(P.x, box[k][3]) && fpi::ge(P.y, box[k][1]) && fpi::le(P.y, box[k][4]) &&
          fpi::ge(P.z, box[k][2]) && fpi::le(P.z, box[k][5]))
        mask |= (1ull << k);
    }
    d.near_mask[p] = mask;
    const unsigned long long v = fpi::bits(sdem::norm3(sdem::xyz(d.vel0[p])));
    const unsigned long long a = fpi::bits(sdem::norm3(sdem::xyz(d.acc0[p])));
    vb = v > vb ? v : vb;
    ab = a > ab ? a : ab;
  }
  __shared__ unsigned long long part[kThreads / 32][2];
  __shared__ int last;
  for (int o = 16; o > 0; o >>= 1) {
    const unsigned long long v = __shfl_down_sync(0xffffffffu, vb, o), a = __shfl_down_sync(0xffffffffu, ab, o);
    vb = v > vb ? v : vb;
    ab = a > ab ? a : ab;
  }
  if ((threadIdx.x & 31) == 0) {
    part[threadIdx.x >> 5][0] = vb;
    part[threadIdx.x >> 5][1] = ab;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    for (int w = 1; w < kThreads / 32; w++) {
      vb = part[w][0] > vb ? part[w][0] : vb;
      ab = part[w][1] > ab ? part[w][1] : ab;
    }
    d.red[2 * blockIdx.x] = vb;
    d.red[2 * blockIdx.x + 1] = ab;
    __threadfence();
    last = atomicAdd(d.ticket, 1) == (int)gridDim.x - 1;
  }
  __syncthreads();
  if (!last || threadIdx.x != 0) return;
  __threadfence();
  *d.ticket = 0;
  // the other blocks' partials, read at L2 (never cached in this SM's L1)
  vb = 0ull;
  ab = 0ull;
  for (int b = 0; b < (int)gridDim.x; b++) {
    const unsigned long long v = __ldcg(&d.red[2 * b]), a = __ldcg(&d.red[2 * b + 1]);
    vb = v > vb ? v : vb;
    ab = a > ab ? a : ab;
  }
  const int it = *d.iter;
  double max_v = fpi::from_bits(vb);
  double max_a = fpi::from_bits(ab);
  max_v = max_v + d.max_wall_vel;
  max_v = (max_v > 0.3) ? max_v : 0.3;
  max_v = max_v * 1.5;
  double gn = sdem::norm3(sdem::mk3(d.g.x, d.g.y, d.g.z));
  max_a = (max_a > gn) ? max_a : gn;
  max_a = max_a * 1.5;
  double t = (sqrt(max_v * max_v + 2.0 * max_a * d.dx1) - max_v) / max_a;
  int numIter = (int)(t / d.law.dt);
  numIter = numIter > 1 ? numIter : 1;
  numIter = numIter < d.wall_max_update_iter ? numIter : d.wall_max_update_iter;
  *d.next_update = it + numIter;
  reset_step_counters(d);
}

// ---------------------------------------------------------------------------
// Periodic images: PC_Comm_For_Cntct (Prtcl_Comm.f90:554-877, y pencil, one
// rank).  Passes in the reference's order -- y (from the locals, up to two
// images each), then +x, -x, +z, -z, each over the images made so far and
// then the locals -- as ordered stream compactions: a flag per candidate
// (images first, then locals), an exclusive scan, a scatter.  Candidate j of
// a pass: j < gcap is image j (if j < ng), j >= gcap is local j - gcap.
enum GhostPass { GP_Y = 0, GP_XP = 1, GP_XM = 2, GP_ZP = 3, GP_ZM = 4 };


// number of images candidate P spawns in this pass
__device__ __forceinline__ int ghost_count(const Dev& d, int pass, const dbl4& P) {
  const double L = d.lencs;
  switch (pass) {
    case GP_Y: return (P.y <= d.dmin.y + L ? 1 : 0) + (P.y >= d.dmax.y - L ? 1 : 0);
    case GP_XP: return P.x >= d.dmax.x - L ? 1 : 0;
    case GP_XM: return (P.x <= d.dmin.x + L && P.x >= d.dmin.x) ? 1 : 0;
    case GP_ZP: return P.z >= d.dmax.z - L ? 1 : 0;
    default: return (P.z <= d.dmin.z + L && P.z >= d.dmin.z) ? 1 : 0;
  }
}

__global__ void k_ghost_flag(Dev d, int pass) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  const int len = d.gcap + d.n_launch;
  if (j >= len) return;
  const int n = *d.n, ng = *d.ng;
  int src = -1;
  if (j < d.gcap) {
    if (pass != GP_Y && j < ng) src = n + j;
  } else if (j - d.gcap < n) {
    src = j - d.gcap;
  }
  d.gflag[j] = src >= 0 ? ghost_count(d, pass, d.posr[src]) : 0;
}

__global__ void k_ghost_scatter(Dev d, int pass) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  const int len = d.gcap + d.n_launch;
  if (j >= len || d.gflag[j] == 0) return;
  const int n = *d.n, ng = *d.ng;
  const int src = j < d.gcap ? n + j : j - d.gcap;
  const dbl4 P = d.posr[src];
  int out = ng + d.goff[j];
  auto emit = [&](int dir, double shift) {
    if (out >= d.gcap) {
      raise(d, SDEM_E_CAPACITY, out);
      return;
    }
    const int g = n + out;
    dbl4 Q = P;
    if (dir == 0) Q.x = P.x + shift;
    else if (dir == 1) Q.y = P.y + shift;
    else Q.z = P.z + shift;
    d.posr[g] = Q;
    d.gid[g] = d.gid[src];
    d.ptype[g] = d.ptype[src];
    d.vel0[g] = d.vel0[src];
    d.rv0[g] = d.rv0[src];
    out++;
  };
  switch (pass) {
    case GP_Y:
      if (P.y <= d.dmin.y + d.lencs) emit(1, d.Lbox.y);
      if (P.y >= d.dmax.y - d.lencs) emit(1, -d.Lbox.y);
      break;
    case GP_XP: emit(0, -d.Lbox.x); break;
    case GP_XM: emit(0, d.Lbox.x); break;
    case GP_ZP: emit(2, -d.Lbox.z); break;
    default: emit(2, d.Lbox.z); break;
  }
}

__global__ void k_ghost_count(Dev d) {
  const int add = d.goff[d.gcap + d.n_launch];
  int ng = *d.ng + add;
  if (ng > d.gcap) ng = d.gcap;
  *d.ng = ng;
  *d.nt = *d.n + ng;
}

// The fourth word of a velocity record carries the particle's id and type
// (low and high 32 bits), so that the force kernel learns both from the
// velocity load it needs anyway instead of two more scattered loads.
__device__ __forceinline__ double id_tag(int gid, int ptype) {
  return __hiloint2double(ptype, gid);
}
__device__ __forceinline__ int tag_gid(double w) { return __double2loint(w); }
__device__ __forceinline__ int tag_type(double w) { return __double2hiint(w); }

__global__ void k_tag_vel(dbl4* __restrict__ vel0, const int* __restrict__ gid, const int* __restrict__ ptype, int n) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) vel0[i].w = id_tag(gid[i], ptype[i]);
}

// Fixed spheres join the search after the images (zero velocities); in the
// within-cell order they rank below every moving sphere and image (the
// reference gives them search indices 1..nFixed, Prtcl_NBS_Munjiza.f90:86).
__global__ void k_fixed_append(Dev d) {
  const int f = blockIdx.x * blockDim.x + threadIdx.x;
  const int base = *d.n + *d.ng;
  if (f == 0) *d.nt = base + d.nfix;
  if (f >= d.nfix) return;
  const int g = base + f;
  d.posr[g] = d.fix_posr[f];
  d.gid[g] = d.fix_gid[f];
  d.ptype[g] = d.fix_ptype[f];
  d.vel0[g] = make_dbl4(0.0, 0.0, 0.0, id_tag(d.fix_gid[f], d.fix_ptype[f]));
  d.rv0[g] = make_dbl4(0.0, 0.0, 0.0, 0.0);
}

// ---------------------------------------------------------------------------
// Binning: NBSM_clcBoxIndex (Prtcl_NBS_Munjiza.f90:193-198) + counting sort.
// Linear cell key orders cells as the reference's sweep visits them:
// row iy (outer), column ix, cell iz (inner).
__global__ void k_bin(Dev d) {
  int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= *d.nt) return;
  const dbl4 P = d.posr[p];
  // the grid of the particle's level (hierarchical search: by type,
  // NBSMH_clcBoxIndex_and_BuildYList, Prtcl_Hrchl_Munjiza.f90:247-336)
  const fpi::Divisor* dc = &d.cdiv;
  float cellf = d.cellf;
  int nx = d.nx, ny = d.ny, nz = d.nz;
  long long base = 0;
  if (d.hier) {
    const LevelGrid& G = d.lv[d.type_lvl[d.ptype[p] - 1]];
    dc = &G.div;
    cellf = G.cellf;
    nx = G.nx; ny = G.ny; nz = G.nz;
    base = G.base;
  }
  // floor((x - x0) / cell_len), the quotient IEEE-rounded, on the integer
  // pipes; the reference's index is this + 1.  The offsets inside the cell
  // become the single-precision prefilter copy.
  int32_t ox, oy, oz;
  const int fx = fpi::floor_div(P.x - d.x0, *dc, nx, ox);
  const int fy = fpi::floor_div(P.y - d.y0, *dc, ny, oy);
  const int fz = fpi::floor_div(P.z - d.z0, *dc, nz, oz);
  if (fx < 0 || fy < 0 || fz < 0) {
    raise(d, SDEM_E_GRID, p);
    d.cell_of[p] = -1;
    return;
  }
  // offset in [0, 1) as a float from its top 23 bits (1.f - 1 is exact; an
  // int-to-float conversion would take the FP64 pipe's rate)
  auto unit = [](int32_t o) { return __uint_as_float(0x3F800000u | ((uint32_t)o >> 8)) - 1.0f; };
  d.pf[p] = make_float4(unit(ox) * cellf, unit(oy) * cellf, unit(oz) * cellf, fpi::to_float_trunc(P.w));
  const long long lkey = ((long long)fy * nx + (long long)fx) * nz + (long long)fz;
  const long long key = base + lkey;
  d.cell_of[p] = (int)key;
  if (d.pcell) d.pcell[p] = make_int4(fx, fy, fz, (int)lkey);
  d.tmp_rank[p] = atomicAdd(&d.cell_cnt[key], 1);
}

__global__ void k_scatter(Dev d) {
  int p = blockIdx.x * blockDim.x + threadIdx.x;
  // this step's owner table starts empty (images never own; the count-only
  // entry point has no table)
  if (d.own_cnt && p < *d.n) d.own_cnt[d.gid[p]] = 0;
  if (p >= *d.nt) return;
  int key = d.cell_of[p];
  if (key < 0) return;
  d.tmp_sorted[d.cell_start[key] + d.tmp_rank[p]] = p;
}

// Deterministic order inside a cell: decreasing particle index (the reference
// pushes Y, X and Z lists front-first, Prtcl_NBS_Munjiza.f90:224-271).
__global__ void k_cellorder(Dev d) {
  int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= *d.nt) return;
  int key = d.cell_of[p];
  if (key < 0) return;
  int a = d.cell_start[key], b = d.cell_start[key + 1];
  // reference search index order: fixed spheres (appended after the moving
  // spheres and images here) come first there, so they rank lowest
  const int moving = d.fix_gid ? *d.n + *d.ng : 0x7FFFFFFF;
  auto ref_key = [&](int q) { return q >= moving ? q - moving : q + d.nfix; };
  const int kp = ref_key(p);
  int rank = 0;
  for (int t = a; t < b; t++) rank += (ref_key(d.tmp_sorted[t]) > kp);
  d.sorted[a + rank] = p;
  d.sortpos[p] = a + rank;
  // single-precision copy relative to the particle's own cell corner (made
  // by the binning)
  d.spos[a + rank] = d.pf[p];
}

// ---------------------------------------------------------------------------
// NBSM_LoopNBSMask + NBSM_FineSearch2 for one target (one thread per sort
// position s).  Visit order per target: the tail of its own cell, then
// (ix,iy,iz-1), (ix-1,iy,iz-1..iz+1), then row iy-1: columns ix-1..ix+1,
// cells iz-1..iz+1 -- the order of Prtcl_NBS_Munjiza.f90:409-468.
// Six blocks per SM (40 registers): the walk is latency bound, and the extra
// resident warps measured faster than the unconstrained 60-register build.
template <bool kHier>
__global__ void __launch_bounds__(kThreads, kSearchBlocksPerSM) k_search(Dev d, int s_begin, int s_end) {
  int s = s_begin + blockIdx.x * blockDim.x + threadIdx.x;
  const int nt = *d.nt;
  const int nloc = *d.n;
  unsigned long long cand = 0, cand_x = 0;
  if (s < s_end) {
    if (s >= nt) {
      d.row_cnt[s] = 0;
    } else {
      const int m = d.sorted[s];
      // a periodic image as target pairs with local particles only
      // (LoopNBSMask, Prtcl_NBS_Munjiza.f90:358-405 -> FineSearch3(n, m))
      const bool m_img = m >= nloc;
      // the target's grid: the base grid, or its level's (hierarchical search)
      int lvl = 0, nx = d.nx, nz = d.nz;
      long long lbase = 0;
      float cellf = d.cellf;
      if (kHier) {
        lvl = d.type_lvl[d.ptype[m] - 1];
        const LevelGrid& G = d.lv[lvl];
        nx = G.nx;
        nz = G.nz;
        lbase = G.base;
        cellf = G.cellf;
      }
      // the target's cell, as the binning found it (in its level's grid)
      const int4 tc = d.pcell[m];
      const int ix = tc.x, iy = tc.y, iz = tc.z, key = tc.w;
      const float4 Pf = d.spos[s];
      const float margin = d.pf_margin;
      int cnt = 0;
      const int K = d.K, Kin = d.Kin, nall = d.nall;
      // The single-precision distance is within pf_margin of the exact one, so
      // outside the band |d - (ri+rj)| < pf_margin the FP32 test decides the
      // reference's FP64 test (NBSM_FineSearch2, Prtcl_NBS_Munjiza.f90:514-522);
      // only candidates inside the band run the FP64 test here.  FP64 work left
      // in this divergent loop would occupy the FP64 pipe with one or two lanes.
      // (ox, oy, oz): target cell corner minus candidate cell corner (0 or one cell)
      auto test = [&](int t, const float4 Qf, float ox, float oy, float oz, unsigned long long& ctr) {
        if (m_img) {
          if (d.sorted[t] >= nloc) return;   // image-image pairs are not searched
          ctr++;
        }
        const float fx = (Pf.x - Qf.x) + ox, fy = (Pf.y - Qf.y) + oy, fz = (Pf.z - Qf.z) + oz;
        const float d2f = fx * fx + fy * fy + fz * fz;
        const float rs = Pf.w + Qf.w;
        const float bhi = rs + margin;
        if (d2f > bhi * bhi) return;
        const int q = d.sorted[t];
        const float blo = rs - margin;
        if (!(d2f < blo * blo)) {
          const dbl4 Pm = d.posr[m], Pq = d.posr[q];
          double dr = Pm.w + Pq.w;
          double dr2 = dr * dr;
          double dx = Pm.x - Pq.x;
          double d2sum = dx * dx;
          if (d2sum > dr2) return;
          double dy = Pm.y - Pq.y;
          d2sum = dy * dy + d2sum;
          if (d2sum > dr2) return;
          double dz = Pm.z - Pq.z;
          d2sum = dz * dz + d2sum;
          if (d2sum > dr2) return;
        }
        if (cnt < K) {
          d.row_partner[(size_t)cnt * nall + s] = q;
          if (q < nloc) {   // an image receives no force: it has no in-list
            int slot = atomicAdd(&d.in_cnt[q], 1);
            if (slot < Kin) d.in_list[(size_t)q * Kin + slot] = ((unsigned)s << 6) | (unsigned)cnt;
            else raise(d, SDEM_E_CL_FULL, q);
          }
        } else {
          raise(d, SDEM_E_CL_FULL, m);
        }
        cnt++;
      };
      // Candidates [a, b) of one range, in order; with SDEM_SEARCH_PREFETCH the
      // next candidate's record is requested (read-only path) before the
      // current one is tested.  In a column (cells iz-1, iz, iz+1 consecutive
      // in the sort) the z offset changes at the inner boundaries z1, z2.
      auto walk = [&](int a, int b, int z1, int z2, float ox, float oy, float oz0, float oz1, float oz2,
                      unsigned long long& ctr) {
#if SDEM_SEARCH_PREFETCH
        if (a >= b) return;
        float4 Qn = __ldg(&d.spos[a]);
        for (int t = a; t < b; t++) {
          const float4 Qf = Qn;
          if (t + 1 < b) Qn = __ldg(&d.spos[t + 1]);
          test(t, Qf, ox, oy, t < z1 ? oz0 : (t < z2 ? oz1 : oz2), ctr);
        }
#else
        for (int t = a; t < b; t++) test(t, d.spos[t], ox, oy, t < z1 ? oz0 : (t < z2 ? oz1 : oz2), ctr);
#endif
      };
      // Cell boundaries of the whole half shell are loaded up front (they do
      // not depend on one another), then the candidates are walked in the
      // reference's order.  The three cells iz-1..iz+1 of one (ix, iy) column
      // are consecutive in the sort, so a column is one range with two inner
      // boundaries; cells outside the grid are empty ranges.
      const int* __restrict__ cs = d.cell_start + lbase;
      const int tail_end = cs[key + 1];
      const int own_lo = iz > 0 ? cs[key - 1] : 0, own_hi = iz > 0 ? cs[key] : 0;   // cell (ix, iy, iz-1)
      int cb[4][4];
      const int ccx[4] = {ix - 1, ix - 1, ix, ix + 1}, ccy[4] = {iy, iy - 1, iy - 1, iy - 1};
#pragma unroll
      for (int c = 0; c < 4; c++) {
        const int cx = ccx[c], cy = ccy[c];
        if (cx < 0 || cx >= nx || cy < 0) {
          cb[c][0] = cb[c][1] = cb[c][2] = cb[c][3] = 0;
        } else {
          const int kb = (cy * nx + cx) * nz + iz;   // the grid holds fewer than 2^31 cells
          cb[c][1] = cs[kb];
          cb[c][2] = cs[kb + 1];
          cb[c][0] = iz > 0 ? cs[kb - 1] : cb[c][1];
          cb[c][3] = iz + 1 < nz ? cs[kb + 2] : cb[c][2];
        }
      }
      // same cell, particles after the target in list order
      walk(s + 1, tail_end, tail_end, tail_end, 0.f, 0.f, 0.f, 0.f, 0.f, cand);
      // (ix, iy, iz-1)
      walk(own_lo, own_hi, own_hi, own_hi, 0.f, 0.f, cellf, cellf, cellf, cand);
      if (!m_img) cand += (unsigned long long)((tail_end - s - 1) + (own_hi - own_lo));
      // columns (ix-1, iy), then (ix-1..ix+1, iy-1), cells iz-1, iz, iz+1
#pragma unroll
      for (int c = 0; c < 4; c++) {
        const float ox = (float)(ix - ccx[c]) * cellf, oy = (float)(iy - ccy[c]) * cellf;
        walk(cb[c][0], cb[c][3], cb[c][1], cb[c][2], ox, oy, cellf, 0.f, -cellf, cand);
        if (!m_img) cand += (unsigned long long)(cb[c][3] - cb[c][0]);
      }
      // Hierarchical search: then the 27 cells around the target's cell in
      // every coarser level, next coarser first (NBSMH_Loop_CrossMask,
      // Prtcl_Hrchl_Munjiza.f90:762-863): the row below, the same row, the
      // row above; columns crs_ix-1..+1; cells crs_iz-1..+1.  Offsets between
      // cell corners are whole target cells (coarse cells are coe fine ones).
      if (kHier) {
        const int mk = d.lv[lvl].mult;
        for (int j = lvl - 1; j >= 0; j--) {
          const LevelGrid& X = d.lv[j];
          const int coe = 1 << (mk - X.mult);
          const int cx0 = ix / coe, cy0 = iy / coe, cz0 = iz / coe;
          const int* __restrict__ csx = d.cell_start + X.base;
          for (int r = -1; r <= 1; r++) {
            const int cy = cy0 + r;
            if (cy < 0 || cy >= X.ny) continue;
            for (int lx = -1; lx <= 1; lx++) {
              const int cx = cx0 + lx;
              if (cx < 0 || cx >= X.nx) continue;
              const int kc = (cy * X.nx + cx) * X.nz;
              const float ox = (float)(ix - cx * coe) * cellf, oy = (float)(iy - cy * coe) * cellf;
              for (int l = -1; l <= 1; l++) {
                const int cz = cz0 + l;
                if (cz < 0 || cz >= X.nz) continue;
                const int a = csx[kc + cz], b = csx[kc + cz + 1];
                const float oz = (float)(iz - cz * coe) * cellf;
                walk(a, b, b, b, ox, oy, oz, oz, oz, cand_x);
                if (!m_img) cand_x += (unsigned long long)(b - a);
              }
            }
          }
        }
      }
      d.row_cnt[s] = cnt < K ? cnt : K;

    }
  }
  for (int o = 16; o > 0; o >>= 1) {
    cand += __shfl_down_sync(0xffffffffu, cand, o);
    cand_x += __shfl_down_sync(0xffffffffu, cand_x, o);
  }
  if ((threadIdx.x & 31) == 0 && cand) atomicAdd(&d.counters[0], cand);
  if ((threadIdx.x & 31) == 0 && cand_x) atomicAdd(&d.counters[9], cand_x);
}

// ---------------------------------------------------------------------------
// The same search on the one-level grid, warp-cooperative and staged through
// shared memory.  A warp takes 32 consecutive target sort positions; the
// targets of one cell form a group and share one candidate list -- the cell
// itself (each target uses the tail after its own position), then the
// reference's half shell in its visit order.  Every lane first loads the
// cell boundaries of its own target's list (the loads of all groups in
// flight at once).  The warp then stages each group's list in shared memory
// with asynchronous copies (cp.async: the candidates' single-precision
// records and particle indices), one group ahead: group g+1's copies travel
// while group g is tested.  One target at a time, the lanes test 32
// consecutive candidates; a ballot over the hits gives every hit its row
// slot in visit order, so rows, in-list keys and counters equal those of the
// thread-per-target walk.  The tests are the same expressions as k_search's
// (the prefilter, then the exact FP64 test inside its band).
constexpr int kSearchWarps = 8;        // warps per block
constexpr int kStage = 96;             // staged candidates per warp and buffer (longer lists go in pieces)
#ifndef SDEM_SEARCH_MIN_BLOCKS
#define SDEM_SEARCH_MIN_BLOCKS 2       // resident blocks per SM the register budget allows
#endif
#ifndef SDEM_SEARCH_WARP
#define SDEM_SEARCH_WARP 0             // 1: the warp-cooperative search on the one-level grid
#endif

__device__ __forceinline__ float corner_offset(int code, float cellf) {
  return code == 1 ? cellf : (code == 2 ? -cellf : 0.f);
}
__device__ __forceinline__ void cp_async16(void* smem, const void* gmem) {
  const unsigned sa = (unsigned)__cvta_generic_to_shared(smem);
  asm volatile("cp.async.ca.shared.global [%0], [%1], 16;\n" ::"r"(sa), "l"(gmem) : "memory");
}
__device__ __forceinline__ void cp_async4(void* smem, const void* gmem) {
  const unsigned sa = (unsigned)__cvta_generic_to_shared(smem);
  asm volatile("cp.async.ca.shared.global [%0], [%1], 4;\n" ::"r"(sa), "l"(gmem) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
__device__ __forceinline__ void cp_async_wait_1() { asm volatile("cp.async.wait_group 1;\n" ::: "memory"); }
__device__ __forceinline__ void cp_async_wait_0() { asm volatile("cp.async.wait_group 0;\n" ::: "memory"); }

// The candidate list of a target cell in visit order: six ranges of sort
// positions (own cell; cell (ix,iy,iz-1); columns (ix-1,iy), (ix-1..ix+1,iy-1),
// each of cells iz-1..iz+1, consecutive in the sort).  Corner offsets
// (target cell corner minus candidate cell corner) per axis are codes
// 0 -> 0, 1 -> +cell, 2 -> -cell, packed x | y << 2 | z << 4; a column's z
// code changes at its inner cell boundaries zb1, zb2.
struct CandList {
  int ra[6], rb[6], zb1[4], zb2[4];
};

__device__ __forceinline__ void cand_list(const int* __restrict__ cs, int key, int ix, int iy, int iz, int nx, int nz,
                                          CandList& L) {
  const int a0 = cs[key];
  L.ra[0] = a0; L.rb[0] = cs[key + 1];
  L.ra[1] = iz > 0 ? cs[key - 1] : 0; L.rb[1] = iz > 0 ? a0 : 0;
#pragma unroll
  for (int c = 0; c < 4; c++) {
    const int cx = c == 0 ? ix - 1 : ix - 2 + c, cy = c == 0 ? iy : iy - 1;
    int b0 = 0, b1 = 0, b2 = 0, b3 = 0;
    if (!(cx < 0 || cx >= nx || cy < 0)) {
      const int kb = (cy * nx + cx) * nz + iz;   // the grid holds fewer than 2^31 cells
      b1 = cs[kb];
      b2 = cs[kb + 1];
      b0 = iz > 0 ? cs[kb - 1] : b1;
      b3 = iz + 1 < nz ? cs[kb + 2] : b2;
    }
    L.ra[2 + c] = b0; L.rb[2 + c] = b3; L.zb1[c] = b1; L.zb2[c] = b2;
  }
}

// the list of lane `src` (all lanes call)
__device__ __forceinline__ void shfl_list(const CandList& mine, int src, CandList& L) {
#pragma unroll
  for (int r = 0; r < 6; r++) {
    L.ra[r] = __shfl_sync(0xffffffffu, mine.ra[r], src);
    L.rb[r] = __shfl_sync(0xffffffffu, mine.rb[r], src);
  }
#pragma unroll
  for (int c = 0; c < 4; c++) {
    L.zb1[c] = __shfl_sync(0xffffffffu, mine.zb1[c], src);
    L.zb2[c] = __shfl_sync(0xffffffffu, mine.zb2[c], src);
  }
}

__device__ __forceinline__ int list_len(const CandList& L) {
  int m = 0;
#pragma unroll
  for (int r = 0; r < 6; r++) m += L.rb[r] - L.ra[r];
  return m;
}

// sort position and corner-offset code of entry i of the list
__device__ __forceinline__ void list_entry(const CandList& L, int i, int& t, int& cd) {
  t = 0;
  cd = 0;
  int base = 0;
#pragma unroll
  for (int r = 0; r < 6; r++) {
    const int len = L.rb[r] - L.ra[r];
    if (i >= base && i < base + len) {
      t = L.ra[r] + (i - base);
      if (r == 1) {
        cd = 1 << 4;
      } else if (r >= 2) {
        const int c = r - 2;
        const int xy = (c <= 1 ? 1 : (c == 2 ? 0 : 2)) | (c == 0 ? 0 : 1) << 2;
        cd = xy | (t < L.zb1[c] ? 1 : (t < L.zb2[c] ? 0 : 2)) << 4;
      }
    }
    base += len;
  }
}

__global__ void __launch_bounds__(kSearchWarps * 32, SDEM_SEARCH_MIN_BLOCKS) k_search_warp(Dev d, int s_begin, int s_end) {
  __shared__ float4 st_q[kSearchWarps][2][kStage];
  __shared__ int st_i[kSearchWarps][2][kStage];
  __shared__ unsigned char st_c[kSearchWarps][2][kStage];
  const unsigned FULL = 0xffffffffu;
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const int s0 = s_begin + (blockIdx.x * kSearchWarps + w) * 32;
  if (s0 >= s_end) return;   // the whole warp
  const int nt = *d.nt, nloc = *d.n;
  const int K = d.K, Kin = d.Kin, nall = d.nall;
  const float margin = d.pf_margin, cellf = d.cellf;
  const int* __restrict__ cs = d.cell_start;
  const int s_me = s0 + lane;
  const bool live = s_me < s_end && s_me < nt;
  if (s_me < s_end && s_me >= nt) d.row_cnt[s_me] = 0;
  int m_me = 0, cnt_me = 0, key_me = -1;
  float4 pf_me = make_float4(0.f, 0.f, 0.f, 0.f);
  CandList mine;
  if (live) {
    m_me = d.sorted[s_me];
    const int4 tc = d.pcell[m_me];
    key_me = tc.w;
    pf_me = d.spos[s_me];
    cand_list(cs, tc.w, tc.x, tc.y, tc.z, d.nx, d.nz, mine);
  } else {
#pragma unroll
    for (int r = 0; r < 6; r++) mine.ra[r] = mine.rb[r] = 0;
#pragma unroll
    for (int c = 0; c < 4; c++) mine.zb1[c] = mine.zb2[c] = 0;
  }
  // live targets are a prefix of the warp's lanes; a group starts where the
  // cell changes (the sort order is the cell order)
  const int nlive = __popc(__ballot_sync(FULL, live));
  const int key_prev = __shfl_up_sync(FULL, key_me, 1);
  unsigned leaders = __ballot_sync(FULL, live && (lane == 0 || key_me != key_prev));
  unsigned long long cand = 0;

  // stage the list of the group led by lane `lead` into buffer `buf` (copies
  // only when it fits; one commit group either way)
  auto stage = [&](int lead, int buf) -> int {
    CandList L;
    shfl_list(mine, lead, L);
    const int M = list_len(L);
    if (M <= kStage) {
      for (int i = lane; i < M; i += 32) {
        int t, cd;
        list_entry(L, i, t, cd);
        cp_async16(&st_q[w][buf][i], &d.spos[t]);
        cp_async4(&st_i[w][buf][i], &d.sorted[t]);
        st_c[w][buf][i] = (unsigned char)cd;
      }
    }
    cp_async_commit();
    return M;
  };

  // test candidates [lo, hi) of the buffer (entry i at i - base) for target lane jj
  auto test_range = [&](int jj, int buf, int base, int lo, int hi) {
    const int s_t = s0 + jj;
    const int m_t = __shfl_sync(FULL, m_me, jj);
    const bool img = m_t >= nloc;
    float4 Pf;
    Pf.x = __shfl_sync(FULL, pf_me.x, jj);
    Pf.y = __shfl_sync(FULL, pf_me.y, jj);
    Pf.z = __shfl_sync(FULL, pf_me.z, jj);
    Pf.w = __shfl_sync(FULL, pf_me.w, jj);
    int cnt_t = __shfl_sync(FULL, cnt_me, jj);
    for (int i0 = lo; i0 < hi; i0 += 32) {
      const int i = i0 + lane;
      bool hit = false;
      int q = 0;
      if (i < hi) {
        const float4 Qf = st_q[w][buf][i - base];
        q = st_i[w][buf][i - base];
        const int cd = st_c[w][buf][i - base];
        if (!img || q < nloc) {   // an image or fixed target pairs with local particles only
          cand++;
          const float ox = corner_offset(cd & 3, cellf), oy = corner_offset((cd >> 2) & 3, cellf),
                      oz = corner_offset((cd >> 4) & 3, cellf);
          const float fx = (Pf.x - Qf.x) + ox, fy = (Pf.y - Qf.y) + oy, fz = (Pf.z - Qf.z) + oz;
          const float d2f = fx * fx + fy * fy + fz * fz;
          const float rs = Pf.w + Qf.w;
          const float bhi = rs + margin;
          if (!(d2f > bhi * bhi)) {
            hit = true;
            const float blo = rs - margin;
            if (!(d2f < blo * blo)) {
              const dbl4 Pm = d.posr[m_t], Pq = d.posr[q];
              double dr = Pm.w + Pq.w;
              double dr2 = dr * dr;
              double dx = Pm.x - Pq.x;
              double d2sum = dx * dx;
              if (d2sum > dr2) hit = false;
              double dy = Pm.y - Pq.y;
              d2sum = dy * dy + d2sum;
              if (d2sum > dr2) hit = false;
              double dz = Pm.z - Pq.z;
              d2sum = dz * dz + d2sum;
              if (d2sum > dr2) hit = false;
            }
          }
        }
      }
      const unsigned mask = __ballot_sync(FULL, hit);
      if (hit) {
        const int slot = cnt_t + __popc(mask & ((1u << lane) - 1u));
        if (slot < K) {
          d.row_partner[(size_t)slot * nall + s_t] = q;
          if (q < nloc) {   // an image receives no force: it has no in-list
            const int is = atomicAdd(&d.in_cnt[q], 1);
            if (is < Kin) d.in_list[(size_t)q * Kin + is] = ((unsigned)s_t << 6) | (unsigned)slot;
            else raise(d, SDEM_E_CL_FULL, q);
          }
        } else {
          raise(d, SDEM_E_CL_FULL, m_t);
        }
      }
      cnt_t += __popc(mask);
    }
    if (lane == jj) cnt_me = cnt_t;
  };

  if (nlive > 0) {
    int lead = __ffs(leaders) - 1;
    leaders &= leaders - 1;
    int M = stage(lead, 0);
    for (int g = 0; lead < nlive; g++) {
      const int buf = g & 1;
      const int next = leaders ? __ffs(leaders) - 1 : nlive;   // the next group's leader ends this group
      int Mn = 0;
      if (leaders) Mn = stage(next, buf ^ 1);
      else cp_async_commit();
      cp_async_wait_1();
      __syncwarp();
      const int a0 = __shfl_sync(FULL, mine.ra[0], lead);
      if (M <= kStage) {
        for (int jj = lead; jj < next; jj++) test_range(jj, buf, 0, s0 + jj - a0 + 1, M);
      } else {
        // a list longer than the buffer: pieces staged with plain loads
        CandList L;
        shfl_list(mine, lead, L);
        for (int pb = 0; pb < M; pb += kStage) {
          const int pe = min(M, pb + kStage);
          for (int i = pb + lane; i < pe; i += 32) {
            int t, cd;
            list_entry(L, i, t, cd);
            st_q[w][buf][i - pb] = d.spos[t];
            st_i[w][buf][i - pb] = d.sorted[t];
            st_c[w][buf][i - pb] = (unsigned char)cd;
          }
          __syncwarp();
          for (int jj = lead; jj < next; jj++) test_range(jj, buf, pb, max(s0 + jj - a0 + 1, pb), pe);
          __syncwarp();
        }
      }
      __syncwarp();
      lead = next;
      if (leaders) leaders &= leaders - 1;
      M = Mn;
    }
    cp_async_wait_0();
  }
  if (live) d.row_cnt[s_me] = cnt_me < K ? cnt_me : K;
  for (int o = 16; o > 0; o >>= 1) cand += __shfl_down_sync(FULL, cand, o);
  if (lane == 0 && cand) atomicAdd(&d.counters[0], cand);
}

// Wall contacts of each particle: FindContactsPW (Prtcl_ContactSearchPW.f90:308-317)
// walks the near-wall list front-first, i.e. the highest wall index first.
// Slots j < kKw per particle keep that order; the compact list feeds k_wall_force.
__global__ void __launch_bounds__(kThreads) k_wall_detect(Dev d) {
  const int m = blockIdx.x * blockDim.x + threadIdx.x;
  int nwc = 0;
  if (m < *d.n) {
    unsigned long long mask = d.near_mask[m];
    if (mask) {
      const dbl4 Pm = d.posr[m];
      const int ncap = d.ncap;
      while (mask) {
        int wi = 63 - __clzll((long long)mask);
        mask &= ~(1ull << wi);
        sdem::Wall W = sdem::load_wall(d.walls, d.wflags, wi);
        double ovrlp;
        r3 nv;
        if (!sdem::wall_contact(W, Pm, ovrlp, nv)) continue;
        if (nwc < kKw) {
          d.w_wall[(size_t)nwc * ncap + m] = wi;
          d.w_geo[(size_t)nwc * ncap + m] = make_dbl4(nv.x, nv.y, nv.z, ovrlp);
          int k = atomicAdd(d.wl_cnt, 1);
          d.wl[k] = (m << 3) | nwc;
        } else {
          raise(d, SDEM_E_CL_FULL, m);
        }
        nwc++;
      }
    }
    const int nw_c = nwc < kKw ? nwc : kKw;
    d.w_cnt[m] = nw_c;
    d.wh_cnt[d.gid[m]] = nw_c;
    int deg = min(d.in_cnt[m], d.Kin) + d.row_cnt[d.sortpos[m]] + nw_c;
    deg = deg < kDegBuckets - 1 ? deg : kDegBuckets - 1;
    d.deg_of[m] = deg;
    // warp-aggregated slot in the bucket: one atomic per distinct degree per warp
    const unsigned act = __activemask();
    const unsigned peers = __match_any_sync(act, deg);
    const int lane = threadIdx.x & 31;
    const int leader = __ffs(peers) - 1;
    int base = 0;
    if (lane == leader) base = atomicAdd(&d.deg_cnt[deg], __popc(peers));
    base = __shfl_sync(peers, base, leader);
    d.deg_rank[m] = base + __popc(peers & ((1u << lane) - 1u));
  }
  for (int o = 16; o > 0; o >>= 1) nwc += __shfl_down_sync(0xffffffffu, nwc, o);
  if ((threadIdx.x & 31) == 0 && nwc) atomicAdd(&d.counters[1], (unsigned long long)nwc);
}

// Gather order: bucket starts (highest degree first; every block scans the
// 64 bucket counts itself), then each particle to its bucket slot.
__global__ void k_degree_scatter(Dev d) {
  static_assert(kDegBuckets == 64, "two buckets per lane of one warp");
  __shared__ int start[kDegBuckets];
  if (threadIdx.x < 32) {
    const int l = threadIdx.x;
    const int b0 = kDegBuckets - 1 - 2 * l, b1 = b0 - 1;
    const int c0 = d.deg_cnt[b0], c1 = d.deg_cnt[b1];
    const int v = c0 + c1;
    int incl = v;
    for (int o = 1; o < 32; o <<= 1) {
      const int t = __shfl_up_sync(0xffffffffu, incl, o);
      if (l >= o) incl += t;
    }
    start[b0] = incl - v;
    start[b1] = incl - v + c0;
  }
  __syncthreads();
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= *d.n) return;
  // what the gather needs first, read here in index order (coalesced, apart
  // from the row of p) and stored at the gather position in one record
  const int s = d.sortpos[p];
  const int nin = min(d.in_cnt[p], d.Kin);
  GRec g;
  g.p = p;
  g.s = s;
  g.own_a = d.row_off[s];
  g.counts = (d.row_cnt[s] << 16) | (nin << 8) | d.w_cnt[p];
  g.r = d.posr[p].w;
  g.pad = 0.0;
  d.gorder[start[d.deg_of[p]] + d.deg_rank[p]] = g;
}

// One thread per wall contact: Find_insert on the particle's bucket (key = wall)
// + ContactForce_PW (Prtcl_CL_and_CF.f90:227-249, 832-856).
__global__ void __launch_bounds__(kThreads) k_wall_force(Dev d) {
  const int nwl = *d.wl_cnt;
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < nwl; k += gridDim.x * blockDim.x) {
    const int e = d.wl[k];
    const int p = e >> 3, j = e & 7;
    const size_t at = (size_t)j * d.ncap + p;
    const int wi = d.w_wall[at];
    const dbl4 geo = d.w_geo[at];
    const int g = d.gid[p];
    dbl4 hist = make_dbl4(0.0, 0.0, 0.0, -2.0);
    const int pc = d.wh_cnt_prev[g];
    for (int i = 0; i < pc; i++)
      if (d.wh_wall_prev[(size_t)g * kKw + i] == wi) { hist = d.wh_hist_prev[(size_t)g * kKw + i]; break; }
    sdem::Wall W = sdem::load_wall(d.walls, d.wflags, wi);
    const double* P = d.bpw + ((size_t)(W.wall_type - 1) * d.nT + (d.ptype[p] - 1)) * SDEM_BP_SIZE;
    const double ri = d.posr[p].w;
    r3 S, M, Mr;
    // "the normal vector points from particle i to j": Norm_v = (-1)*nv (:849-851)
    r3 Norm_v = sdem::scale3(sdem::mk3(geo.x, geo.y, geo.z), -1.0);
    sdem::force_law(d.law, P, sdem::xyz(d.vel0[p]), W.vel, sdem::xyz(d.rv0[p]), sdem::mk3(0.0, 0.0, 0.0), ri,
                    1.00E20 * ri, Norm_v, geo.w, hist, S, M, Mr);
    d.w_S[at] = sdem::d4(S, 0.0);
    d.w_M[at] = sdem::d4(M, 0.0);   // Moment (the gather scales it by ri)
    d.w_Mr[at] = sdem::d4(Mr, 0.0);
    d.wh_wall[(size_t)g * kKw + j] = wi;
    d.wh_hist[(size_t)g * kKw + j] = hist;
  }
}

// Each contact's row (its target's sort position) for the rows [s_begin, s_end),
// so that the one-thread-per-contact force kernel reads its row instead of
// searching the row offsets.
__global__ void k_row_fill(Dev d, int s_begin, int s_end) {
  const int s = s_begin + blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= s_end) return;
  const int a = d.row_off[s], k = d.row_cnt[s];
  for (int j = 0; j < k; j++)
    if (a + j < d.ccap) d.c_row[a + j] = s;
}

// ---------------------------------------------------------------------------
// One thread per contact: Find_insert's history lookup + ContactForce_PP.
// Contacts of the rows [s_begin, s_end).  kOneSided: the search holds periodic
// images or fixed spheres (pairs whose force goes to one sphere only).
template <bool kOneSided>
__global__ void __launch_bounds__(kThreads, SDEM_FORCE_MIN_BLOCKS) k_force(Dev d, int s_begin, int s_end) {
  const int nloc = *d.n;
  const int c0 = d.row_off[s_begin], C = d.row_off[s_end];
  if (C > d.ccap) {
    if (blockIdx.x == 0 && threadIdx.x == 0) raise(d, SDEM_E_CL_FULL, C);
    return;
  }
  unsigned long long nimg = 0, nfx = 0;
  const int first_fixed = nloc + *d.ng;   // search index of the first fixed sphere
  for (int c = c0 + blockIdx.x * blockDim.x + threadIdx.x; c < C; c += gridDim.x * blockDim.x) {
    const int s = d.c_row[c];
    const int slot = c - d.row_off[s];
    int m = d.sorted[s];
    int q = d.row_partner[(size_t)slot * d.nall + s];
    // both particles' state records; the velocity records carry id and type
    const dbl4 Pm = d.posr[m], Pq = d.posr[q];
    const dbl4 Vm = d.vel0[m], Vq = d.vel0[q], Wm = d.rv0[m], Wq = d.rv0[q];
    const int gm = tag_gid(Vm.w), gq = tag_gid(Vq.w);
    // particle-particle (AddContactPP) or local-image (AddContactPPG) pair; the
    // lower id is particle i of the force law either way
    // (Prtcl_NBS_Munjiza.f90:525-529, Prtcl_CL_and_CF.f90:773-797)
    const bool img = kOneSided && ((m >= nloc) || (q >= nloc));
    const bool m_loc = m < nloc;              // the local particle of an image pair is m
    const int oth = m_loc ? q : m;
    const bool m_lo = gm < gq;
    // Find_insert's bucket: the lower id's for PP, the local particle's for PPG
    const int owner = img ? (m_loc ? gm : gq) : (m_lo ? gm : gq);
    const int partner = img ? (m_loc ? gq : gm) : (m_lo ? gq : gm);
    const dbl4 Pi = m_lo ? Pm : Pq, Pj = m_lo ? Pq : Pm;
    const dbl4 Vi = m_lo ? Vm : Vq, Vj = m_lo ? Vq : Vm;
    const dbl4 Wi = m_lo ? Wm : Wq, Wj = m_lo ? Wq : Wm;
    // Prtcl_BnryProp(pType(lower id), pType(higher id)) for PP (:743),
    // (pType(local), pType(image)) for PPG (:772)
    const int tm = tag_type(Vm.w), tq = tag_type(Vq.w);
    const int ta = img ? (m_loc ? tm : tq) : (m_lo ? tm : tq);
    const int tb = img ? (m_loc ? tq : tm) : (m_lo ? tq : tm);
    dbl4 hist = make_dbl4(0.0, 0.0, 0.0, -2.0);
    {
      const int2* oe = d.own_c_prev + (size_t)owner * d.Ko;
      // the first entry is read beside the count (the table always holds Ko
      // entries per owner; an entry past the count is not used)
      const int2 e0 = oe[0];
      const int k = d.own_cnt_prev[owner];
      if (k > 0 && e0.y == partner) {
        hist = d.c_hist_prev[e0.x];
      } else {
        for (int j = 1; j < k; j++) {
          const int2 e = oe[j];
          if (e.y == partner) { hist = d.c_hist_prev[e.x]; break; }
        }
      }
    }
    const double* P = d.bpp + ((size_t)(tb - 1) * d.nT + (ta - 1)) * SDEM_BP_SIZE;
    // Norm_v = Posj .nv. Posi (real4_nv, Prtcl_TypeDef.f90:268-281) and
    // ovrlp = dr - sqrt(d2sum) (NBSM_FineSearch2/3, Prtcl_NBS_Munjiza.f90:514-522)
    // share one length: d2sum = dz*dz + (dy*dy + dx*dx) is bitwise
    // (sx*sx + sy*sy) + sz*sz for s = Posj - Posi (squares ignore the sign and
    // a two-term IEEE sum is commutative).
    const r3 sv = sdem::sub3(sdem::xyz(Pj), sdem::xyz(Pi));
    const double normv = sdem::norm3(sv);
    const double ovrlp = (Pi.w + Pj.w) - normv;
    r3 Norm_v = fpi::gt(normv, 1.0000E-10) ? sdem::div3(sv, normv) : sdem::mk3(0.0, 0.0, 0.0);
    r3 S, M, Mr;
    sdem::force_law(d.law, P, sdem::xyz(Vi), sdem::xyz(Vj), sdem::xyz(Wi), sdem::xyz(Wj), Pi.w, Pj.w, Norm_v, ovrlp,
                    hist, S, M, Mr);
    d.c_ogid[c] = owner | (img ? kImgFlag : 0);
    d.c_pgid[c] = partner;
    d.c_hist[c] = hist;
    // signed for the row's target: it adds S and Mr when it is particle i and
    // subtracts them when it is j (x - y == x + (-y): the sign goes on the
    // bits); the partner adds their negations
    const uint64_t sg = m_lo ? 0ull : fpi::kSign;
    auto flip = [sg](double v) { return fpi::from_bits(fpi::bits(v) ^ sg); };
    ContactRec& rec = d.c_rec[c];
    rec.S = make_dbl4(flip(S.x), flip(S.y), flip(S.z), 0.0);
    rec.M = sdem::d4(M, 0.0);   // Moment: each side's gather scales it by its own radius
    rec.Mr = make_dbl4(flip(Mr.x), flip(Mr.y), flip(Mr.z), 0.0);
    const int os = atomicAdd(&d.own_cnt[owner], 1);
    if (os < d.Ko) d.own_c[(size_t)owner * d.Ko + os] = make_int2(c, partner);
    else raise(d, SDEM_E_CL_FULL, owner);
    // one-sided pairs: with an image (AddContactPPG) or a fixed sphere (AddContactPPFix)
    if (kOneSided) {
      const bool fx = img && oth >= first_fixed;
      nimg += (img && !fx) ? 1ull : 0ull;
      nfx += fx ? 1ull : 0ull;
    }
  }
  if (kOneSided) {
    for (int o = 16; o > 0; o >>= 1) {
      nimg += __shfl_down_sync(0xffffffffu, nimg, o);
      nfx += __shfl_down_sync(0xffffffffu, nfx, o);
    }
    if ((threadIdx.x & 31) == 0 && nimg) atomicAdd(&d.counters[5], nimg);
    if ((threadIdx.x & 31) == 0 && nfx) atomicAdd(&d.counters[8], nfx);
  }
}

// ---------------------------------------------------------------------------
// Per particle: contact sums in the reference's scatter order, walls,
// acceleration and Adams-Bashforth update.
//
// Order: the reference adds each pair's force to both particles when the pair
// is visited.  Pairs that hold particle p are visited (a) as the partner of an
// earlier target of p's own cell, (b) as p's own target row, (c) as the partner
// of targets in later cells; (a) and (c) are ordered by (target sort position,
// slot), which is exactly the packed in-list key, and (b) is the row order.
// Sorts v[0..N) ascending with a bitonic network (constant indices: registers).
template <int N>
__device__ __forceinline__ void sort_net(unsigned (&v)[N]) {
#pragma unroll
  for (int k = 2; k <= N; k <<= 1)
#pragma unroll
    for (int j = k >> 1; j > 0; j >>= 1)
#pragma unroll
      for (int i = 0; i < N; i++) {
        const int l = i ^ j;
        if (l > i) {
          const unsigned a = v[i], b = v[l];
          const unsigned lo = a < b ? a : b, hi = a < b ? b : a;
          if ((i & k) == 0) { v[i] = lo; v[l] = hi; }
          else { v[i] = hi; v[l] = lo; }
        }
      }
}

__global__ void __launch_bounds__(kThreads) k_gather(Dev d) {
  const int tid = blockIdx.x * blockDim.x + threadIdx.x;
  if (tid >= *d.n) return;
  const GRec gr = d.gorder[tid];
  const int p = gr.p, s = gr.s;
  const int ncap = d.ncap;
  const double rp = gr.r;
  r3 F = sdem::mk3(0.0, 0.0, 0.0), T = sdem::mk3(0.0, 0.0, 0.0);

  // The contact records of p in the reference's scatter order: in-list
  // entries of earlier targets, p's own row, in-list entries of later
  // targets, then wall contacts.  Their indices go to a small per-thread list
  // first (integer work), so the FP64 additions run in one loop whose trip
  // count is the warp's maximum, not once per branch.
  const int own_a = gr.own_a, own_n = gr.counts >> 16;
  const int nin = (gr.counts >> 8) & 0xFF;
  const int nwc = gr.counts & 0xFF;
  // entry: (contact index << 1) | (p is the row's target), or -(wall slot + 1)
  int list[2 * kMaxK + kKw];
  int nl = 0;
  auto push_in = [&](unsigned key) { list[nl++] = (d.row_off[key >> 6] + (int)(key & 63u)) << 1; };
  auto push_own = [&]() {
    for (int j = 0; j < own_n; j++) list[nl++] = ((own_a + j) << 1) | 1;
  };
  if (nin <= 8) {
    unsigned u[8];
#pragma unroll
    for (int k = 0; k < 8; k++) u[k] = k < nin ? d.in_list[(size_t)p * d.Kin + k] : 0xffffffffu;
    sort_net<8>(u);
#pragma unroll
    for (int k = 0; k < 8; k++)
      if (k < nin && (int)(u[k] >> 6) < s) push_in(u[k]);
    push_own();
#pragma unroll
    for (int k = 0; k < 8; k++)
      if (k < nin && (int)(u[k] >> 6) > s) push_in(u[k]);
  } else if (nin <= 16) {
    unsigned u[16];
#pragma unroll
    for (int k = 0; k < 16; k++) u[k] = k < nin ? d.in_list[(size_t)p * d.Kin + k] : 0xffffffffu;
    sort_net<16>(u);
#pragma unroll
    for (int k = 0; k < 16; k++)
      if (k < nin && (int)(u[k] >> 6) < s) push_in(u[k]);
    push_own();
#pragma unroll
    for (int k = 0; k < 16; k++)
      if (k < nin && (int)(u[k] >> 6) > s) push_in(u[k]);
  } else {
    unsigned e[kMaxK];
    for (int k = 0; k < nin; k++) {
      unsigned v = d.in_list[(size_t)p * d.Kin + k];
      int j = k - 1;
      while (j >= 0 && e[j] > v) { e[j + 1] = e[j]; j--; }
      e[j + 1] = v;
    }
    int k = 0;
    for (; k < nin && (int)(e[k] >> 6) < s; k++) push_in(e[k]);
    push_own();
    for (; k < nin; k++) push_in(e[k]);
  }
  for (int j = 0; j < nwc; j++) list[nl++] = -(j + 1);

  for (int k = 0; k < nl; k++) {
    const int e = list[k];
    const int c = e >= 0 ? (e >> 1) : e;
    const bool tgt = e < 0 || (e & 1);   // a wall record or p's own row: as stored
    dbl4 S, Ms, Mr;
    if (c >= 0) {
      const ContactRec& rec = d.c_rec[c];
      S = rec.S;
      Ms = rec.M;
      Mr = rec.Mr;
    } else {
      const size_t at = (size_t)(-c - 1) * ncap + p;
      S = d.w_S[at];
      Ms = d.w_M[at];
      Mr = d.w_Mr[at];
    }
    // F(pid) + (Fnij+Ftij) / F(pjd) - (Fnij+Ftij);
    // T + r*Moment + Mrij / T + r*Moment - Mrij  (Prtcl_ContactForce_inc.f90:69-86).
    // The records are signed for the row's target; the partner adds their
    // negations (x - y is x + (-y) in IEEE arithmetic), so that every lane
    // runs the same FP64 additions.
    const uint64_t sg = tgt ? 0ull : fpi::kSign;
    auto flip = [sg](double v) { return fpi::from_bits(fpi::bits(v) ^ sg); };
    F = sdem::add3(F, sdem::mk3(flip(S.x), flip(S.y), flip(S.z)));
    // r*Moment with p's own radius (ri*Moment or rj*Moment of the reference)
    T = sdem::add3(sdem::add3(T, sdem::scale3(sdem::xyz(Ms), rp)), sdem::mk3(flip(Mr.x), flip(Mr.y), flip(Mr.z)));
  }
  d.F[p] = sdem::d4(F, 0.0);
  d.T[p] = sdem::d4(T, 0.0);
}

// Per particle: clc_Acceleration, Prtcl_Integrate and the periodic wrap /
// out-of-domain flag.  The state records a particle's update reads (the
// rotational history after the linear).
enum IntField { IF_POSR, IF_F, IF_T, IF_V0, IF_W0, IF_TH, IF_V1, IF_A1, IF_V2, IF_A2, IF_W1, IF_AL1, IF_W2, IF_AL2,
                IF_N };

__device__ __forceinline__ const dbl4* int_src(const Dev& d, int f) {
  switch (f) {
    case IF_POSR: return d.posr;
    case IF_F: return d.F;
    case IF_T: return d.T;
    case IF_V0: return d.vel0;
    case IF_W0: return d.rv0;
    case IF_TH: return d.theta;
    case IF_V1: return d.vel1;
    case IF_A1: return d.acc1;
    case IF_V2: return d.vel2;
    case IF_A2: return d.acc2;
    case IF_W1: return d.rv1;
    case IF_AL1: return d.ra1;
    case IF_W2: return d.rv2;
    default: return d.ra2;
  }
}

// get(f) returns the particle's record of field f (from shared memory or HBM)
template <class Get>
__device__ __forceinline__ void integrate_body(const Dev& d, const int p, const Get& get) {
  const dbl4 Pp = get(IF_POSR);
  const r3 F = sdem::xyz(get(IF_F)), T = sdem::xyz(get(IF_T));
  const dbl4 v1 = get(IF_V0);
  const dbl4 w1 = get(IF_W0);
  const int ti = tag_type(v1.w);

  // clc_Acceleration, Prtcl_DEMSystem.f90:174-180
  // F/Mass and T/Inertia (IEEE quotients)
  const double Mass = d.mass[ti - 1], Inertia = d.inertia[ti - 1];
  r3 a1 = sdem::add3(sdem::div3(F, Mass),
                     sdem::mk3(d.g.x, d.g.y, d.g.z));
  r3 al1 = sdem::div3(T, Inertia);
  const double dt = d.law.dt;
  const double AB2C1 = 3.0 / 2.0;
  // AB2's second coefficient is -1/2: v * (-1/2) is exact, an exponent
  // decrement on the integer pipe instead of a multiplication on the FP64 pipe
  auto nh3 = [](r3 v) { return sdem::mk3(fpi::mul_neg_half(v.x), fpi::mul_neg_half(v.y), fpi::mul_neg_half(v.z)); };
  const double AB3C1 = 23.0 / 12.0, AB3C2 = -16.0 / 12.0, AB3C3 = 5.0 / 12.0;

  // Prtcl_Integrate, linear part (Prtcl_Integration.f90:25-53)
  r3 x = sdem::xyz(Pp);
  r3 lv1 = sdem::xyz(v1);
  r3 lv1_new;
  if (d.pi == SDEM_PIM_FE) {
    x = sdem::add3(x, sdem::scale3(lv1, dt));
    lv1_new = sdem::add3(lv1, sdem::scale3(a1, dt));
    d.acc0[p] = sdem::d4(a1, 0.0);
  } else if (d.pi == SDEM_PIM_AB2) {
    r3 lv2 = sdem::xyz(get(IF_V1));
    r3 la2 = sdem::xyz(get(IF_A1));
    x = sdem::add3(x, sdem::scale3(sdem::add3(sdem::scale3(lv1, AB2C1), nh3(lv2)), dt));
    lv1_new = sdem::add3(lv1, sdem::scale3(sdem::add3(sdem::scale3(a1, AB2C1), nh3(la2)), dt));
    d.vel1[p] = sdem::d4(lv1, 0.0);
    d.acc1[p] = sdem::d4(a1, 0.0);
    d.acc0[p] = sdem::d4(a1, 0.0);
  } else {
    r3 lv2 = sdem::xyz(get(IF_V1)), lv3 = sdem::xyz(get(IF_V2));
    r3 la2 = sdem::xyz(get(IF_A1)), la3 = sdem::xyz(get(IF_A2));
    x = sdem::add3(x, sdem::scale3(sdem::add3(sdem::add3(sdem::scale3(lv1, AB3C1), sdem::scale3(lv2, AB3C2)),
                                              sdem::scale3(lv3, AB3C3)), dt));
    lv1_new = sdem::add3(lv1, sdem::scale3(sdem::add3(sdem::add3(sdem::scale3(a1, AB3C1), sdem::scale3(la2, AB3C2)),
                                                      sdem::scale3(la3, AB3C3)), dt));
    d.vel2[p] = sdem::d4(lv2, 0.0);
    d.vel1[p] = sdem::d4(lv1, 0.0);
    d.acc2[p] = sdem::d4(la2, 0.0);
    d.acc1[p] = sdem::d4(a1, 0.0);
    d.acc0[p] = sdem::d4(a1, 0.0);
  }
  d.vel0[p] = sdem::d4(lv1_new, v1.w);   // keeps the id/type word
  d.posr[p] = sdem::d4(x, Pp.w);

  // rotational part (Prtcl_Integration.f90:55-86)
  r3 th = sdem::xyz(get(IF_TH));
  r3 rw1 = sdem::xyz(w1);
  if (d.pri == SDEM_PIM_FE) {
    th = sdem::add3(th, sdem::scale3(rw1, dt));
    d.rv0[p] = sdem::d4(sdem::add3(rw1, sdem::scale3(al1, dt)), 0.0);
    d.ra0[p] = sdem::d4(al1, 0.0);
  } else if (d.pri == SDEM_PIM_AB2) {
    // Prtcl_Integration.f90:64 starts from GPrtcl_linVel(1,i), already updated
    r3 wa = d.quirk ? lv1_new : rw1;
    r3 rw2 = sdem::xyz(get(IF_W1));
    r3 ra2 = sdem::xyz(get(IF_AL1));
    th = sdem::add3(th, sdem::scale3(sdem::add3(sdem::scale3(wa, AB2C1), nh3(rw2)), dt));
    d.rv0[p] = sdem::d4(sdem::add3(wa, sdem::scale3(sdem::add3(sdem::scale3(al1, AB2C1), nh3(ra2)), dt)), 0.0);
    d.rv1[p] = sdem::d4(wa, 0.0);
    d.ra1[p] = sdem::d4(al1, 0.0);
    d.ra0[p] = sdem::d4(al1, 0.0);
  } else {
    r3 rw2 = sdem::xyz(get(IF_W1)), rw3 = sdem::xyz(get(IF_W2));
    r3 ra2 = sdem::xyz(get(IF_AL1)), ra3 = sdem::xyz(get(IF_AL2));
    th = sdem::add3(th, sdem::scale3(sdem::add3(sdem::add3(sdem::scale3(rw1, AB3C1), sdem::scale3(rw2, AB3C2)),
                                                sdem::scale3(rw3, AB3C3)), dt));
    d.rv0[p] = sdem::d4(sdem::add3(rw1, sdem::scale3(sdem::add3(sdem::add3(sdem::scale3(al1, AB3C1), sdem::scale3(ra2, AB3C2)),
                                                                sdem::scale3(ra3, AB3C3)), dt)), 0.0);
    d.rv2[p] = sdem::d4(rw2, 0.0);
    d.rv1[p] = sdem::d4(rw1, 0.0);
    d.ra2[p] = sdem::d4(ra2, 0.0);
    d.ra1[p] = sdem::d4(al1, 0.0);
    d.ra0[p] = sdem::d4(al1, 0.0);
  }
  d.theta[p] = sdem::d4(th, 0.0);

  // Comm_For_Exchange, y pencil, one rank (Prtcl_Comm.f90:1569-1840): a periodic
  // direction wraps the position (passes y, +x, -x, +z, -z); the others delete
  // what left [min, max), in the delete passes (k_finish).
  if (d.per[0] || d.per[1] || d.per[2]) {
    dbl4 Q = sdem::d4(x, Pp.w);
    if (d.per[1]) {
      if (fpi::ge(Q.y, d.dmax.y)) Q.y = Q.y - d.Lbox.y;
      else if (fpi::lt(Q.y, d.dmin.y)) Q.y = Q.y + d.Lbox.y;
    }
    if (d.per[0]) {
      if (fpi::ge(Q.x, d.dmax.x)) Q.x = Q.x - d.Lbox.x;
      if (fpi::lt(Q.x, d.dmin.x)) Q.x = Q.x + d.Lbox.x;
    }
    if (d.per[2]) {
      if (fpi::ge(Q.z, d.dmax.z)) Q.z = Q.z - d.Lbox.z;
      if (fpi::lt(Q.z, d.dmin.z)) Q.z = Q.z + d.Lbox.z;
    }
    d.posr[p] = Q;
    x = sdem::xyz(Q);
  }
  if ((!d.per[1] && (fpi::ge(x.y, d.dmax.y) || fpi::lt(x.y, d.dmin.y))) ||
      (!d.per[0] && (fpi::ge(x.x, d.dmax.x) || fpi::lt(x.x, d.dmin.x))) ||
      (!d.per[2] && (fpi::ge(x.z, d.dmax.z) || fpi::lt(x.z, d.dmin.z)))) {
    int k2 = atomicAdd(d.out_cnt, 1);
    if (k2 < kOutCap) d.out_list[k2] = p;
    else raise(d, SDEM_E_CAPACITY, p);
  }
}

// The update in index order, one thread per particle (coalesced records).
__global__ void __launch_bounds__(kThreads) k_integrate(Dev d) {
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= *d.n) return;
  integrate_body(d, p, [&](int f) { return int_src(d, f)[p]; });
}

// ---------------------------------------------------------------------------
// One-rank delete of particles outside [min,max), y pencil, five passes of
// swap-with-last (Prtcl_Comm.f90:1569-1840).  Single thread; runs on the few
// candidates only (positions of untouched particles equal their index).
__device__ __forceinline__ bool out_pass(const Dev& d, int id, int pass) {
  dbl4 P = d.posr[id];
  if (d.per[pass == 0 ? 1 : (pass <= 2 ? 0 : 2)]) return false;   // wrapped, not deleted
  switch (pass) {
    case 0: return P.y >= d.dmax.y || P.y < d.dmin.y;
    case 1: return P.x >= d.dmax.x;
    case 2: return P.x < d.dmin.x;
    case 3: return P.z >= d.dmax.z;
    default: return P.z < d.dmin.z;
  }
}

__device__ void delete_serial(const Dev& d) {
  int U = *d.out_cnt;
  d.moves[0] = 0;
  if (U == 0) return;
  if (U > kOutCap) return;  // already raised
  int* L = d.out_list;
  for (int i = 1; i < U; i++) {  // ascending original index
    int v = L[i], j = i - 1;
    while (j >= 0 && L[j] > v) { L[j + 1] = L[j]; j--; }
    L[j + 1] = v;
  }
  int n = *d.n;
  int nm = 0;  // map: position -> particle (original index) for touched positions
  auto content = [&](int pos) -> int {
    for (int j = nm - 1; j >= 0; j--)
      if (d.map_pos[j] == pos) return d.map_id[j];
    return pos;
  };
  auto set = [&](int pos, int id) {
    for (int j = nm - 1; j >= 0; j--)
      if (d.map_pos[j] == pos) { d.map_id[j] = id; return; }
    d.map_pos[nm] = pos;
    d.map_id[nm] = id;
    nm++;
  };
  auto where = [&](int id) -> int {  // current position of a candidate, -1 if gone
    for (int j = nm - 1; j >= 0; j--)
      if (d.map_id[j] == id && d.map_pos[j] < n) return d.map_pos[j];
    if (id < n && content(id) == id) return id;
    return -1;
  };
  int* B = d.moves + 1 + 2 * (5 * kOutCap);  // scratch after the move list
  for (int pass = 0; pass < 5; pass++) {
    int nb = 0;
    for (int i = 0; i < U; i++) {
      int id = L[i];
      if (!out_pass(d, id, pass)) continue;
      int pos = where(id);
      if (pos < 0) continue;
      int j = nb - 1;
      while (j >= 0 && B[j] > pos) { B[j + 1] = B[j]; j--; }
      B[j + 1] = pos;
      nb++;
    }
    for (int i = 0; i < nb; i++) {
      int b = B[i];
      if (b >= n) break;
      while (true) {
        int v = content(n - 1);
        if (b != n - 1) set(b, v);
        n--;
        if (b >= n) break;
        if (!out_pass(d, v, pass)) break;
      }
    }
  }
  int mv = 0;
  for (int j = 0; j < nm; j++)
    if (d.map_pos[j] < n && d.map_id[j] != d.map_pos[j]) {
      d.moves[1 + 2 * mv] = d.map_pos[j];
      d.moves[2 + 2 * mv] = d.map_id[j];
      mv++;
    }
  d.moves[0] = mv;
  *d.n = n;
}

// GL_copy + CL_copy + CSPW_copy for each move (force and torque are not part of
// GL_copy and stay where they are).  Sources lie beyond the new count and
// destinations below it, so the copies are independent.
__device__ void apply_moves(const Dev& d, int first, int stride) {
  int mv = d.moves[0];
  for (int i = first; i < mv; i += stride) {
    int dst = d.moves[1 + 2 * i], src = d.moves[2 + 2 * i];
    d.gid[dst] = d.gid[src];
    d.ptype[dst] = d.ptype[src];
    d.usrmark[dst] = d.usrmark[src];
    d.posr[dst] = d.posr[src];
    d.vel0[dst] = d.vel0[src];
    d.acc0[dst] = d.acc0[src];
    if (d.tsize > 1) { d.vel1[dst] = d.vel1[src]; d.acc1[dst] = d.acc1[src]; }
    if (d.tsize > 2) { d.vel2[dst] = d.vel2[src]; d.acc2[dst] = d.acc2[src]; }
    d.theta[dst] = d.theta[src];
    d.rv0[dst] = d.rv0[src];
    d.ra0[dst] = d.ra0[src];
    if (d.rsize > 1) { d.rv1[dst] = d.rv1[src]; d.ra1[dst] = d.ra1[src]; }
    if (d.rsize > 2) { d.rv2[dst] = d.rv2[src]; d.ra2[dst] = d.ra2[src]; }
    d.near_mask[dst] = d.near_mask[src];
  }
}

// Self-test of the integer-pipe arithmetic against the hardware instructions:
// operand pairs from a counter-based generator in five families (random bit
// patterns, the physics range, perfect squares and neighbours, exact
// quotients and neighbours, grid coordinates near cell edges).
__device__ __forceinline__ unsigned long long splitmix(unsigned long long z) {
  z += 0x9E3779B97F4A7C15ull;
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}
__device__ __forceinline__ bool same_bits(double a, double b) {
  return __double_as_longlong(a) == __double_as_longlong(b) || (a != a && b != b);
}
__global__ void k_selftest_fp64(long long n, unsigned long long seed, unsigned long long* bad) {
  unsigned long long nb = 0;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    const unsigned long long r0 = splitmix(seed ^ (unsigned long long)i), r1 = splitmix(r0), r2 = splitmix(r1);
    unsigned long long ua, ub;
    switch (i % 5) {
      case 0: ua = r0; ub = r1; break;
      case 1: {
        const unsigned long long ea = 983 + r2 % 60, eb = 983 + (r2 >> 8) % 60;
        ua = ((r2 >> 20) & 1ull) << 63 | ea << 52 | (r0 & fpi::kMant);
        ub = ((r2 >> 21) & 1ull) << 63 | eb << 52 | (r1 & fpi::kMant);
        break;
      }
      case 2: {
        const unsigned long long k = (r0 >> 38) | 1ull;
        const double sq = (double)k * (double)k;
        ua = (unsigned long long)__double_as_longlong(sq) + (r2 % 5) - 2;
        ub = (unsigned long long)__double_as_longlong((double)k);
        break;
      }
      case 3: {
        const unsigned long long m1 = (r0 >> 40) | 1ull, m2 = (r1 >> 40) | 1ull;
        ua = (unsigned long long)__double_as_longlong((double)m1 * (double)m2) + (r2 % 3) - 1;
        ub = (unsigned long long)__double_as_longlong((double)m2);
        break;
      }
      default: {
        const double cell = 1.2e-3 * (1.0 + (double)(r2 % 1000) * 1e-4);
        const double x = ((double)(long long)(r0 % 4000) - 100.0) * cell + ((double)(r1 % 2001) - 1000.0) * 1e-19;
        ua = (unsigned long long)__double_as_longlong(x);
        ub = (unsigned long long)__double_as_longlong(cell);
      }
    }
    const double x = __longlong_as_double((long long)ua), y = __longlong_as_double((long long)ub);
    bool ok = same_bits(fpi::sqrt_rn(x), __dsqrt_rn(x)) && same_bits(fpi::div_rn(x, y), __ddiv_rn(x, y)) &&
              same_bits(fpi::div_rn(y, x), __ddiv_rn(y, x)) &&
              same_bits(fpi::mul_neg_half(x), __dmul_rn(x, -0.5)) && fpi::gt(x, y) == (x > y) &&
              fpi::ge(x, y) == (x >= y) && fpi::lt(x, y) == (x < y) && fpi::le(x, y) == (x <= y);
    const double q = __ddiv_rn(x, y), f = floor(q);
    const int want = (f >= 0.0 && f < 4000.0) ? (int)f : -1;
    ok = ok && fpi::floor_in_range(q, 4000) == want;
    int32_t off = 0;
    const int kq = fpi::floor_div(x, fpi::divisor(y), 4000, off);
    ok = ok && kq == want;
    if (kq >= 0 && fabs(q) < 0x1p26) ok = ok && fabs((double)off * 0x1p-31 - (q - (double)kq)) <= 0x1p-26;
    nb += ok ? 0ull : 1ull;
  }
  if (nb) atomicAdd(bad, nb);
}

// FP64 pipe probe: eight independent DFMA chains per thread, so issue, not
// latency, limits the rate.  The result is written only when it is zero
// (never, for these operands), which keeps the chains alive.
__global__ void __launch_bounds__(256) k_probe_dfma(long long iters, double b, double c, double* sink) {
  double a0 = threadIdx.x * 1e-3 + 1.0, a1 = a0 + 0.1, a2 = a0 + 0.2, a3 = a0 + 0.3;
  double a4 = a0 + 0.4, a5 = a0 + 0.5, a6 = a0 + 0.6, a7 = a0 + 0.7;
  for (long long i = 0; i < iters; i++) {
    a0 = __fma_rn(a0, b, c); a1 = __fma_rn(a1, b, c); a2 = __fma_rn(a2, b, c); a3 = __fma_rn(a3, b, c);
    a4 = __fma_rn(a4, b, c); a5 = __fma_rn(a5, b, c); a6 = __fma_rn(a6, b, c); a7 = __fma_rn(a7, b, c);
  }
  const double s = ((a0 + a1) + (a2 + a3)) + ((a4 + a5) + (a6 + a7));
  if (s == 0.0) sink[blockIdx.x] = s;
}

// Contact snapshot (asynchronous output): the records of the last step and
// each particle's wall records, frozen so that later steps may run while the
// copy travels to the host.
struct SnapContacts {
  int* scal;        // [0] particles, [1] particle-particle records
  int *gid, *og, *pg;
  dbl4* hs;
  int *wcnt, *wwall;  // per particle index: wall record count, kKw wall indices
  dbl4* whist;        // per particle index: kKw wall records
};

__global__ void k_snap_contacts(Dev d, const int* __restrict__ pgid, const dbl4* __restrict__ hist,
                                const int* __restrict__ whc, const int* __restrict__ whw,
                                const dbl4* __restrict__ whh, SnapContacts out, int nall_launch) {
  const int n = *d.n;
  const int C = nall_launch >= 0 ? d.row_off[nall_launch] : 0;   // -1: no step since upload
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    out.scal[0] = n;
    out.scal[1] = C;
  }
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < C || i < n; i += gridDim.x * blockDim.x) {
    if (i < C) {
      out.og[i] = d.c_ogid[i];
      out.pg[i] = pgid[i];
      out.hs[i] = hist[i];
    }
    if (i < n) {
      const int g = d.gid[i];
      out.gid[i] = g;
      const int k = whc[g];
      out.wcnt[i] = k;
      for (int j = 0; j < kKw; j++) {
        out.wwall[(size_t)i * kKw + j] = j < k ? whw[(size_t)g * kKw + j] : -1;
        out.whist[(size_t)i * kKw + j] = j < k ? whh[(size_t)g * kKw + j] : make_dbl4(0.0, 0.0, 0.0, 0.0);
      }
    }
  }
}

// Copies a contact snapshot to (mapped) host memory: exactly the records it holds.
__global__ void k_snap_copy(SnapContacts src, SnapContacts dst) {
  const int n = src.scal[0], C = src.scal[1];
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    dst.scal[0] = n;
    dst.scal[1] = C;
  }
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < C || i < n; i += gridDim.x * blockDim.x) {
    if (i < C) {
      dst.og[i] = src.og[i];
      dst.pg[i] = src.pg[i];
      dst.hs[i] = src.hs[i];
    }
    if (i < n) {
      dst.gid[i] = src.gid[i];
      dst.wcnt[i] = src.wcnt[i];
      for (int j = 0; j < kKw; j++) {
        dst.wwall[(size_t)i * kKw + j] = src.wwall[(size_t)i * kKw + j];
        dst.whist[(size_t)i * kKw + j] = src.whist[(size_t)i * kKw + j];
      }
    }
  }
}

// Upload checks on the device: ids in 1..max_gid and unique (a flag per id),
// types in 1..nT.  status[0] = first error, status[1] = its particle index.
__global__ void k_check_upload(const int* __restrict__ id, const int* __restrict__ ptype, int n, int max_gid, int nT,
                               int* __restrict__ flag, int* __restrict__ status) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int g = id[i];
  int code = 0;
  if (g < 1 || g > max_gid) code = SDEM_E_BAD_ID;
  else if (atomicExch(&flag[g], 1) != 0) code = SDEM_E_BAD_ID + 100;   // duplicate
  else if (ptype[i] < 1 || ptype[i] > nT) code = SDEM_E_ARG;
  if (code && atomicCAS(status, 0, code) == 0) status[1] = i;
}

// Host layout <-> device layout of the per-particle 3-vectors: the ABI's
// [(i*levels + k)*3 + c] doubles against one 32-byte record per particle and
// level.  A null source writes zeros.
__global__ void k_unpack3(dbl4* __restrict__ dst, const double* __restrict__ src, int n, int levels, int k) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  if (!src) {
    dst[i] = make_dbl4(0.0, 0.0, 0.0, 0.0);
    return;
  }
  const double* v = src + ((size_t)i * levels + k) * 3;
  dst[i] = make_dbl4(v[0], v[1], v[2], 0.0);
}

__global__ void k_pack3(double* __restrict__ dst, const dbl4* __restrict__ src, int n, int levels, int k) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const dbl4 a = src[i];
  double* v = dst + ((size_t)i * levels + k) * 3;
  v[0] = a.x;
  v[1] = a.y;
  v[2] = a.z;
}

// Ends a step: the counters of the step (CL and search logs), running sums and
// per-step resets.
__device__ void step_end_serial(const Dev& d, int* counters_out) {
  // every value first (the loads issue together), then the stores
  const int C = d.row_off[d.nall_launch];
  const unsigned long long cnsv = d.counters[0], pw = d.counters[1], ppg = d.counters[5], fx = d.counters[8],
                           cross = d.counters[9];
  const int n = *d.n, it = *d.iter + 1, next = *d.next_update;
  const int pp = C - (int)ppg - (int)fx;
  counters_out[SDEM_CNT_PP] = pp;
  counters_out[SDEM_CNT_PPG] = (int)ppg;
  counters_out[SDEM_CNT_PPFIX] = (int)fx;
  counters_out[SDEM_CNT_PW] = (int)pw;
  counters_out[SDEM_CNT_CNSV] = (int)cnsv;
  counters_out[SDEM_CNT_NLOCAL] = n;
  *d.iter = it;
  counters_out[SDEM_CNT_ITER] = it;
  counters_out[SDEM_CNT_NEXTWALL] = next;
  counters_out[SDEM_CNT_CNSV_CROSS] = (int)cross;
  d.counters[2] += (unsigned long long)pp;
  d.counters[3] += pw;
  d.counters[4] += 1ull;
  d.counters[0] = 0;
  d.counters[1] = 0;
  d.counters[5] = 0;
  d.counters[8] = 0;
  d.counters[9] = 0;
  *d.out_cnt = 0;
  *d.wl_cnt = 0;
}

// The end of a step in one block: the serial delete passes (thread 0), the
// moves they imply (all threads), the counters (thread 0), then a copy of the
// device scalars (status, particle count, counters) into mapped host memory,
// one word per thread, so that the host reads them after a stream
// synchronisation without another copy.  Two mirror slots, by the parity of
// the new iteration number: a step's copy survives while the next step runs.
__global__ void k_finish(Dev d, int* counters_out, const int* scal, int* mirror, int nscal) {
  if (threadIdx.x == 0) delete_serial(d);
  __syncthreads();
  apply_moves(d, threadIdx.x, blockDim.x);
  __syncthreads();
  if (threadIdx.x == 0) step_end_serial(d, counters_out);
  __syncthreads();
  if (mirror && threadIdx.x < nscal) {
    int* slot = mirror + (*d.iter & 1) * nscal;
    slot[threadIdx.x] = scal[threadIdx.x];
  }
}

// ---------------------------------------------------------------------------
// Allocation-free contact count (sdem_count_contacts_noalloc).
//
// Callers that cannot allocate device memory -- a host that runs inside
// another framework's memory pool, or code between a pool reset and its next
// allocation -- can still count the contacts of a particle set they already
// hold on the device, e.g. to size their contact buffers before creating a
// handle.  The scratch this needs (search grid, counting sort, prefilter copy)
// is a file-scope device array of fixed size: every GPU that loads the library
// holds it, ~7.3 MB, until the process exits.
constexpr int kNaMaxN = 1 << 16;       // SDEM_NOALLOC_MAX_PARTICLES
constexpr int kNaMaxCells = 1 << 19;   // SDEM_NOALLOC_MAX_CELLS
constexpr int kNaBlocks = (kNaMaxCells + kScanTile - 1) / kScanTile;
struct NoAllocScratch {
  int cell_cnt[kNaMaxCells];
  int cell_start[kNaMaxCells + 1];
  int cell_of[kNaMaxN];
  int tmp_rank[kNaMaxN];
  int tmp_sorted[kNaMaxN];
  int sorted[kNaMaxN];
  int sortpos[kNaMaxN];
  float4 spos[kNaMaxN];
  float4 pf[kNaMaxN];
  int bsum[kNaBlocks];
  int n;
  int status[2];
  unsigned long long counts[2];   // exact contacts, candidate pairs
};
static __device__ __align__(256) NoAllocScratch g_noalloc_scratch;

__global__ void k_na_begin(NoAllocScratch* S, int n) {
  S->n = n;
  S->status[0] = 0;
  S->status[1] = 0;
  S->counts[0] = 0ull;
  S->counts[1] = 0ull;
}

// The search of k_search without its rows: the same half shell, the same
// single-precision decision with the FP64 test in the ambiguous band; it only
// counts numCntcts(1) and num_Cnsv_cntct.  Only the sort positions this call
// wrote are searched: a particle outside the grid (SDEM_E_GRID) is not placed,
// so sorted[cell_start[ncell] .. n) still holds an earlier call's indices,
// which may lie beyond this call's d_posR.  After a binning error nothing is
// searched at all.
__global__ void __launch_bounds__(kThreads) k_na_count(Dev d, unsigned long long* counts) {
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  unsigned long long cand = 0, hits = 0;
  const int placed = d.cell_start[d.ncell];
  if (d.status[0] == 0 && s < *d.n && s < placed) {
    const int m = d.sorted[s];
    const int key = d.cell_of[m];
    const int iz = key % d.nz;
    const int rest = key / d.nz;
    const int ix = rest % d.nx;
    const int iy = rest / d.nx;
    const float4 Pf = d.spos[s];
    const dbl4 Pm = d.posr[m];
    const float margin = d.pf_margin;
    auto test = [&](int t, float ox, float oy, float oz) {
      const float4 Qf = d.spos[t];
      const float fx = (Pf.x - Qf.x) + ox, fy = (Pf.y - Qf.y) + oy, fz = (Pf.z - Qf.z) + oz;
      const float d2f = fx * fx + fy * fy + fz * fz;
      const float rs = Pf.w + Qf.w;
      const float bhi = rs + margin;
      if (d2f > bhi * bhi) return;
      const float blo = rs - margin;
      if (!(d2f < blo * blo)) {
        const dbl4 Pq = d.posr[d.sorted[t]];
        double dr = Pm.w + Pq.w;
        double dr2 = dr * dr;
        double dx = Pm.x - Pq.x;
        double d2sum = dx * dx;
        if (d2sum > dr2) return;
        double dy = Pm.y - Pq.y;
        d2sum = dy * dy + d2sum;
        if (d2sum > dr2) return;
        double dz = Pm.z - Pq.z;
        d2sum = dz * dz + d2sum;
        if (d2sum > dr2) return;
      }
      hits++;
    };
    {
      const int b = d.cell_start[key + 1];
      for (int t = s + 1; t < b; t++) test(t, 0.f, 0.f, 0.f);
      cand += (unsigned long long)(b - s - 1);
    }
    auto visit = [&](int cx, int cy, int cz) {
      if (cx < 0 || cx >= d.nx || cy < 0 || cz < 0 || cz >= d.nz) return;
      const long long k2 = ((long long)cy * d.nx + cx) * d.nz + cz;
      const int a = d.cell_start[k2], b = d.cell_start[k2 + 1];
      const float ox = (float)(ix - cx) * d.cellf, oy = (float)(iy - cy) * d.cellf, oz = (float)(iz - cz) * d.cellf;
        for (int t = a; t < b; t++) test(t, ox, oy, oz);
      cand += (unsigned long long)(b - a);
    };
    visit(ix, iy, iz - 1);
    visit(ix - 1, iy, iz - 1);
    visit(ix - 1, iy, iz);
    visit(ix - 1, iy, iz + 1);
    for (int lx = -1; lx <= 1; lx++)
      for (int i = -1; i <= 1; i++) visit(ix + lx, iy - 1, iz + i);
  }
  for (int o = 16; o > 0; o >>= 1) {
    cand += __shfl_down_sync(0xffffffffu, cand, o);
    hits += __shfl_down_sync(0xffffffffu, hits, o);
  }
  if ((threadIdx.x & 31) == 0) {
    if (hits) atomicAdd(&counts[0], hits);
    if (cand) atomicAdd(&counts[1], cand);
  }
}

__global__ void k_na_end(const NoAllocScratch* S, unsigned long long* out) {
  out[0] = S->counts[0];
  out[1] = S->counts[1];
}

// ---------------------------------------------------------------------------
// host side
struct Buf {
  void* p = nullptr;
  size_t bytes = 0;
};

}  // namespace

struct sdem_h {
  sdem_cfg cfg{};
  int dev = 0;
  int num_sms = 152;
  cudaStream_t stream = nullptr;
  std::string err;
  std::vector<void*> allocs;
  // tables
  int nT = 0, nWT = 0;
  double maxR = 0.0;
  std::vector<double> h_radius;
  double *radius = nullptr, *mass = nullptr, *inertia = nullptr, *bpp = nullptr, *bpw = nullptr;
  int nw = 0;
  double* walls = nullptr;
  int* wflags = nullptr;
  std::vector<int> h_wall_id;
  double max_wall_vel = 0.0;
  bool have_types = false;
  // grid
  double cell = 0, x0 = 0, y0 = 0, z0 = 0;
  int nx = 0, ny = 0, nz = 0;
  long long ncell = 0;
  int *cell_cnt = nullptr, *cell_start = nullptr, *scan_tmp = nullptr;
  size_t scan_tmp_n = 0;
  // particles
  int n_host = 0;  // count at upload (upper bound of the device count)
  int *gid = nullptr, *ptype = nullptr, *usrmark = nullptr;
  dbl4 *posr = nullptr, *vel[3] = {}, *acc[3] = {}, *theta = nullptr, *rv[3] = {}, *ra[3] = {};
  dbl4 *F = nullptr, *T = nullptr;
  unsigned long long* near_mask = nullptr;
  int *cell_of = nullptr, *tmp_rank = nullptr, *tmp_sorted = nullptr, *sorted = nullptr, *sortpos = nullptr;
  int K = 24;
  int *row_cnt = nullptr, *row_partner = nullptr, *row_off = nullptr, *in_cnt = nullptr;
  unsigned* in_list = nullptr;
  int ccap = 0;
  int *c_ogid = nullptr, *c_pgid[2] = {}, *own_cnt[2] = {}, *c_row = nullptr;
  int2* own_c[2] = {};
  int nall = 0, gcap = 0;
  int fcap = 0, nfix = 0;
  bool hier = false;
  int nlvl = 0;
  LevelGrid lv[kMaxLevels] = {};
  int* type_lvl = nullptr;
  int *fix_gid = nullptr, *fix_ptype = nullptr;
  dbl4* fix_posr = nullptr;
  int *gflag = nullptr, *goff = nullptr;
  // particle-particle records as uploaded (reported until the first step):
  // owner id, partner id, listed under the partner too
  struct UpRec { int owner, partner; bool both; dbl4 hist; };
  std::vector<UpRec> h_up;
  dbl4* c_hist[2] = {};
  ContactRec* c_rec = nullptr;
  int *wh_cnt[2] = {}, *wh_wall[2] = {};
  dbl4* wh_hist[2] = {};
  int *w_cnt = nullptr, *w_wall = nullptr, *wl = nullptr;
  dbl4 *w_geo = nullptr, *w_S = nullptr, *w_M = nullptr, *w_Mr = nullptr;
  float4* spos = nullptr;
  float4* pf = nullptr;
  int4* pcell = nullptr;
  float pf_margin = 0.f;
  int *deg_cnt = nullptr, *deg_of = nullptr, *deg_rank = nullptr;
  GRec* gorder = nullptr;
  // second stream and events of the chunked search/force pipeline
  cudaStream_t stream2 = nullptr;
  cudaEvent_t ev_fork = nullptr, ev_join = nullptr, ev_rows = nullptr, ev_chunk[kMaxChunks] = {};
  int nchunk = kChunks;                  // launch shape (sdem_set_launch); results do not depend on it
  int force_bps = kForceBlocksPerSM;
  int first_pct = 0;                     // percent of the targets in the first chunk (0: whole search waves)
  int cur = 0;  // buffer written by the next step
  // device scalars
  int* scal = nullptr;  // n, status[2], iter, next_update, out_cnt, counters_out[8]
  // device counters: [0] candidates, [1] wall contacts, [2..4] sums since
  // upload, [5] image pairs, [6..7] max |v|, |a| reductions, [8] fixed pairs,
  // [9] cross-level candidates
  unsigned long long* ull = nullptr;
  unsigned long long* red_part = nullptr;   // k_step_begin's per-block maxima
  int *out_list = nullptr, *moves = nullptr, *map_pos = nullptr, *map_id = nullptr;
  int* h_counters = nullptr;  // pinned
  // mapped host copy of the device scalars, written by every step's last
  // kernel; valid while no host write to the scalars came after the last step
  int* h_mirror = nullptr;   // 2 slots of S_SIZE ints, by iteration parity
  int* h_chk = nullptr;      // page-locked: the upload's id/type check (status, detail)
  int* d_mirror = nullptr;
  bool mirror_ok = false;
  long long iter_host = 0;   // device iteration number after the last enqueued step
  cudaEvent_t ev_step[2] = {};   // completion of the step that ends on an iteration of this parity
  long long ev_iter[2] = {-1, -1};   // the iteration each event marks
  double* stage = nullptr;    // device staging of host-layout 3-vectors (upload, download)
  size_t stage_n = 0;
  // asynchronous output: a frozen copy of the state and contacts on the device,
  // downloaded on the I/O stream while later steps run
  cudaStream_t stream_io = nullptr;
  cudaEvent_t ev_snap = nullptr, ev_snap_done = nullptr;
  cudaEvent_t ev_xfer[6] = {};   // upload/download: one staged field copied / packed
  bool snap_busy = false, snap_done = false, snap_contacts = false, snap_stepped = false;
  double* sn_state = nullptr;    // device: posR, 3-vector fields, F, T (host layouts)
  int* sn_ints = nullptr;        // device: id, ptype, usrmark, n
  void* sn_cdev = nullptr;       // device contact snapshot (SnapContacts layout)
  void* sn_chost = nullptr;      // mapped pinned host copy of it
  SnapContacts sn_dev{}, sn_host{}, sn_host_dptr{};
  int* sn_n_host = nullptr;      // pinned
  std::vector<UpRec> sn_up;
  bool stepped = false;
  // two consecutive steps captured as one CUDA graph (the contact buffers
  // alternate every step, so two steps return to the same buffer parity)
  cudaGraphExec_t graph2 = nullptr;
  cudaGraphExec_t graph1[2] = {};   // one step, by the buffer parity it starts from
  long long graph1_launches = 0;
  int graph_cur = -1;       // buffer parity the graph starts from
  long long graph_launches = 0;
  long long graph_gen = 0;   // bumped whenever captured step graphs become invalid
  bool use_graphs = true;
  // diagnostics: kernel launches issued, optional per-phase CUDA events
  long long launches = 0;
  bool prof = false;
  int prof_steps = 0, prof_cap = 0;
  std::vector<cudaEvent_t> prof_ev;   // prof_cap * (kPhases + 1)
};

namespace {

int set_err(sdem_h* h, int code, const std::string& msg) {
  h->err = msg;
  return code;
}

int cuda_fail(sdem_h* h, cudaError_t e, const char* where) {
  return set_err(h, SDEM_E_CUDA, std::string(where) + ": " + cudaGetErrorString(e));
}

#define CK(call)                                   \
  do {                                             \
    cudaError_t e_ = (call);                       \
    if (e_ != cudaSuccess) return cuda_fail(h, e_, #call); \
  } while (0)

template <class T>
int dalloc(sdem_h* h, T** p, size_t count) {
  void* q = nullptr;
  size_t bytes = std::max<size_t>(count, 1) * sizeof(T);
  cudaError_t e = cudaMalloc(&q, bytes);
  if (e != cudaSuccess) {
    cudaGetLastError();
    return set_err(h, SDEM_E_NOMEM, std::string("cudaMalloc of ") + std::to_string(bytes) + " bytes failed");
  }
  cudaMemsetAsync(q, 0, bytes, h->stream);
  h->allocs.push_back(q);
  *p = (T*)q;
  return 0;
}

// Grows the staging buffer to hold `count` doubles (upload/download only).
int ensure_stage(sdem_h* h, size_t count) {
  if (count <= h->stage_n) return 0;
  if (h->stage) {
    cudaStreamSynchronize(h->stream);
    cudaFree(h->stage);
    h->stage = nullptr;
    h->stage_n = 0;
  }
  void* q = nullptr;
  cudaError_t e = cudaMalloc(&q, count * sizeof(double));
  if (e != cudaSuccess) {
    cudaGetLastError();
    return set_err(h, SDEM_E_NOMEM, "cudaMalloc of the upload/download staging buffer failed");
  }
  h->stage = (double*)q;
  h->stage_n = count;
  return 0;
}

enum { S_N = 0, S_STATUS = 1, S_ITER = 3, S_NEXT = 4, S_OUTCNT = 5, S_WLCNT = 6, S_NG = 7, S_COUNTERS = 8,  // counters: 8..16
       S_NT = 20, S_TICKET = 21, S_SIZE = 24 };

Dev make_dev(sdem_h* h) {
  Dev d{};
  const sdem_cfg& c = h->cfg;
  d.ncap = c.n_capacity;
  d.n_launch = h->n_host;
  d.n = h->scal + S_N;
  d.nall = h->nall;
  d.gcap = h->gcap;
  d.nall_launch = h->n_host + h->gcap + h->nfix;
  d.nfix = h->nfix;
  d.hier = h->hier ? 1 : 0;
  d.nlvl = h->nlvl;
  for (int k = 0; k < kMaxLevels; k++) d.lv[k] = h->lv[k];
  d.type_lvl = h->type_lvl;
  d.fix_gid = h->fix_gid;
  d.fix_ptype = h->fix_ptype;
  d.fix_posr = h->fix_posr;
  d.ng = h->scal + S_NG;
  d.nt = h->scal + S_NT;
  d.ticket = h->scal + S_TICKET;
  for (int k = 0; k < 3; k++) d.per[k] = c.periodic[k];
  d.Lbox = make_double3(c.dom_max[0] - c.dom_min[0], c.dom_max[1] - c.dom_min[1], c.dom_max[2] - c.dom_min[2]);
  d.lencs = h->cell;
  d.dmin = make_double3(c.dom_min[0], c.dom_min[1], c.dom_min[2]);
  d.dmax = make_double3(c.dom_max[0], c.dom_max[1], c.dom_max[2]);
  d.gflag = h->gflag;
  d.goff = h->goff;
  d.max_gid = c.max_gid;
  d.K = h->K;
  d.Kin = h->K;
  d.ccap = h->ccap;
  d.tsize = c.tsize;
  d.rsize = c.rsize;
  d.pi = c.pi_method;
  d.pri = c.pri_method;
  d.quirk = c.quirk_ab2_rot;
  d.law.cf_type = c.cf_type;
  d.law.ct_model = c.ct_model;
  d.law.dt = c.dt;
  d.g = make_double3(c.gravity[0], c.gravity[1], c.gravity[2]);
  d.cell = h->cell;
  d.x0 = h->x0;
  d.y0 = h->y0;
  d.z0 = h->z0;
  d.nx = h->nx;
  d.ny = h->ny;
  d.nz = h->nz;
  d.ncell = h->ncell;
  d.dmin = make_double3(c.dom_min[0], c.dom_min[1], c.dom_min[2]);
  d.dmax = make_double3(c.dom_max[0], c.dom_max[1], c.dom_max[2]);
  d.nT = h->nT;
  d.nWT = h->nWT;
  d.radius = h->radius;
  d.mass = h->mass;
  d.inertia = h->inertia;
  d.bpp = h->bpp;
  d.bpw = h->bpw;
  d.nw = h->nw;
  d.walls = h->walls;
  d.wflags = h->wflags;
  d.dx1 = h->maxR * c.wall_neighbor_ratio;
  d.dx2 = h->maxR * (c.wall_neighbor_ratio + 1.0);
  d.max_wall_vel = h->max_wall_vel;
  d.wall_max_update_iter = c.wall_max_update_iter;
  d.gid = h->gid;
  d.ptype = h->ptype;
  d.usrmark = h->usrmark;
  d.posr = h->posr;
  d.vel0 = h->vel[0];
  d.vel1 = h->vel[1];
  d.vel2 = h->vel[2];
  d.acc0 = h->acc[0];
  d.acc1 = h->acc[1];
  d.acc2 = h->acc[2];
  d.theta = h->theta;
  d.rv0 = h->rv[0];
  d.rv1 = h->rv[1];
  d.rv2 = h->rv[2];
  d.ra0 = h->ra[0];
  d.ra1 = h->ra[1];
  d.ra2 = h->ra[2];
  d.F = h->F;
  d.T = h->T;
  d.near_mask = h->near_mask;
  d.cell_of = h->cell_of;
  d.cell_cnt = h->cell_cnt;
  d.cell_start = h->cell_start;
  d.tmp_rank = h->tmp_rank;
  d.tmp_sorted = h->tmp_sorted;
  d.sorted = h->sorted;
  d.sortpos = h->sortpos;
  d.spos = h->spos;
  d.pf = h->pf;
  d.pcell = h->pcell;
  d.cdiv = fpi::divisor(h->cell);
  d.deg_cnt = h->deg_cnt;
  d.deg_of = h->deg_of;
  d.deg_rank = h->deg_rank;
  d.gorder = h->gorder;
  d.pf_margin = h->pf_margin;
  d.cellf = (float)h->cell;
  d.w_cnt = h->w_cnt;
  d.w_wall = h->w_wall;
  d.w_geo = h->w_geo;
  d.w_S = h->w_S;
  d.w_M = h->w_M;
  d.w_Mr = h->w_Mr;
  d.wl = h->wl;
  d.wl_cnt = h->scal + S_WLCNT;
  d.row_cnt = h->row_cnt;
  d.row_partner = h->row_partner;
  d.row_off = h->row_off;
  d.in_cnt = h->in_cnt;
  d.in_list = h->in_list;
  int cu = h->cur, pv = 1 - h->cur;
  d.c_ogid = h->c_ogid;
  d.c_pgid = h->c_pgid[cu];
  d.c_pgid_prev = h->c_pgid[pv];
  d.c_hist = h->c_hist[cu];
  d.c_hist_prev = h->c_hist[pv];
  d.c_rec = h->c_rec;
  d.Ko = h->K;
  d.c_row = h->c_row;
  d.own_cnt = h->own_cnt[cu];
  d.own_c = h->own_c[cu];
  d.own_cnt_prev = h->own_cnt[pv];
  d.own_c_prev = h->own_c[pv];
  d.wh_cnt = h->wh_cnt[cu];
  d.wh_wall = h->wh_wall[cu];
  d.wh_hist = h->wh_hist[cu];
  d.wh_cnt_prev = h->wh_cnt[pv];
  d.wh_wall_prev = h->wh_wall[pv];
  d.wh_hist_prev = h->wh_hist[pv];
  d.status = h->scal + S_STATUS;
  d.counters = h->ull;
  d.red = h->red_part;
  d.iter = h->scal + S_ITER;
  d.next_update = h->scal + S_NEXT;
  d.out_cnt = h->scal + S_OUTCNT;
  d.out_list = h->out_list;
  d.moves = h->moves;
  d.map_pos = h->map_pos;
  d.map_id = h->map_id;
  return d;
}

int grid_for(long long n) { return (int)std::max<long long>(1, (n + kThreads - 1) / kThreads); }

void scan(sdem_h* h, const int* in, long long n, int* out, const int* offset = nullptr) {
  int nb = (int)std::max<long long>(1, (n + kScanTile - 1) / kScanTile);
  k_scan_reduce<<<nb, kScanThreads, 0, h->stream>>>(in, n, h->scan_tmp);
  k_scan_blocks<<<1, 1024, 0, h->stream>>>(h->scan_tmp, nb);
  k_scan_apply<<<nb, kScanThreads, 0, h->stream>>>(in, n, h->scan_tmp, out, offset);
}

int enqueue_step(sdem_h* h) {
  Dev d = make_dev(h);
  int n = h->n_host;
  cudaStream_t st = h->stream;
  cudaEvent_t* ev = nullptr;
  if (h->prof && h->prof_steps < h->prof_cap) ev = &h->prof_ev[(size_t)h->prof_steps * (kPhases + 1)];
  auto mark = [&](int ph) {
    if (ev) cudaEventRecord(ev[ph], st);
  };
  long long L = 0;
  mark(PH_WALL);
  // the refresh schedule (Next_iter_update) advances with or without walls
  k_step_begin<<<h->num_sms * kBeginBlocksPerSM, kThreads, 0, st>>>(d);
  L += 1;
  mark(PH_BIN);
  const int na = n + h->gcap + h->nfix;   // search arrays: locals, periodic images, fixed spheres
  if (h->gcap > 0) {
    const int per[3] = {h->cfg.periodic[0], h->cfg.periodic[1], h->cfg.periodic[2]};
    const int passes[5] = {GP_Y, GP_XP, GP_XM, GP_ZP, GP_ZM};
    const int pdir[5] = {1, 0, 0, 2, 2};
    for (int k = 0; k < 5; k++) {
      if (!per[pdir[k]]) continue;
      k_ghost_flag<<<grid_for(na), kThreads, 0, st>>>(d, passes[k]);
      scan(h, h->gflag, na, h->goff);
      k_ghost_scatter<<<grid_for(na), kThreads, 0, st>>>(d, passes[k]);
      k_ghost_count<<<1, 1, 0, st>>>(d);
      L += 6;
    }
  }
  if (h->nfix > 0) {
    k_fixed_append<<<grid_for(h->nfix), kThreads, 0, st>>>(d);
    L += 1;
  }
  cudaMemsetAsync(h->cell_cnt, 0, sizeof(int) * (size_t)h->ncell, st);
  cudaMemsetAsync(h->in_cnt, 0, sizeof(int) * (size_t)std::max(n, 1), st);
  k_bin<<<grid_for(na), kThreads, 0, st>>>(d);
  mark(PH_SCAN_CELLS);
  scan(h, h->cell_cnt, h->ncell, h->cell_start);
  mark(PH_SCATTER);
  k_scatter<<<grid_for(na), kThreads, 0, st>>>(d);
  mark(PH_CELLORDER);
  k_cellorder<<<grid_for(na), kThreads, 0, st>>>(d);
  mark(PH_SEARCH);
  // Chunked pipeline: the searches of all chunks, then wall detection and wall
  // forces, run on the second stream; each chunk's row offsets (continuing
  // the previous chunk's total), contact rows and forces run on the main
  // stream as soon as its search is done.  Profiling runs one chunk on one
  // stream, so that every phase has its own events.
  const int nchunk = ev ? 1 : h->nchunk;
  cudaStream_t s2 = ev ? st : h->stream2;
  // chunk boundaries on scan tiles, so that each chunk's row scan moves whole
  // aligned tiles
  // The first chunk's search runs alone, before any force: by default it
  // takes as many whole waves of resident search blocks as fit in an even
  // share, when that trims the share by a quarter at most, so that its last
  // wave is full (a partial last wave takes a whole wave's time); or
  // first_pct percent of the targets.  The other chunks share the rest
  // evenly.
  long long first = -1;
  if (nchunk > 1) {
    const long long wave = (long long)h->num_sms * kSearchBlocksPerSM * kThreads;
    const long long share = na / nchunk, whole = share / wave * wave;
    if (h->first_pct > 0) first = (long long)na * h->first_pct / 100;
    else if (whole > 0 && 4 * (share - whole) <= share) first = whole;
  }
  auto cut = [&](int k) {
    if (k == 0) return 0;
    if (k == nchunk) return na;
    const long long c = first < 0 ? (long long)na * k / nchunk : first + (na - first) * (k - 1) / (nchunk - 1);
    return (int)(c & ~(long long)(kScanTile - 1));
  };
  if (s2 != st) {
    cudaEventRecord(h->ev_fork, st);
    cudaStreamWaitEvent(s2, h->ev_fork, 0);
  }
  for (int k = 0; k < nchunk; k++) {
    const int a = cut(k), b = cut(k + 1);
    if (h->hier) k_search<true><<<grid_for(std::max(b - a, 1)), kThreads, 0, s2>>>(d, a, b);
    else if (!SDEM_SEARCH_WARP) k_search<false><<<grid_for(std::max(b - a, 1)), kThreads, 0, s2>>>(d, a, b);
    else {
      const long long warps = (std::max(b - a, 1) + 31) / 32;
      k_search_warp<<<(int)((warps + kSearchWarps - 1) / kSearchWarps), kSearchWarps * 32, 0, s2>>>(d, a, b);
    }
    if (s2 != st) cudaEventRecord(h->ev_chunk[k], s2);
  }
  k_wall_detect<<<grid_for(n), kThreads, 0, s2>>>(d);
  if (s2 == st) {
    mark(PH_SCAN_ROWS);
    scan(h, h->row_cnt, na, h->row_off);
    mark(PH_ROW_FILL);
    k_row_fill<<<grid_for(na), kThreads, 0, st>>>(d, 0, na);
    mark(PH_FORCE);
    if (h->gcap > 0 || h->nfix > 0) k_force<true><<<h->num_sms * 8, kThreads, 0, st>>>(d, 0, na);
    else k_force<false><<<h->num_sms * 8, kThreads, 0, st>>>(d, 0, na);
    mark(PH_WALL_FORCE);
    k_wall_force<<<std::max(1, h->num_sms * 2), kThreads, 0, st>>>(d);
  } else {
    k_wall_force<<<std::max(1, h->num_sms * 2), kThreads, 0, s2>>>(d);
    for (int k = 0; k < nchunk; k++) {
      const int a = cut(k), b = cut(k + 1);
      cudaStreamWaitEvent(st, h->ev_chunk[k], 0);
      scan(h, h->row_cnt + a, b - a, h->row_off + a, k ? h->row_off + a : nullptr);
      if (k == nchunk - 1) {
        // every row offset is known: the gather order (which needs them and
        // the wall contacts, not the forces) is built on the second stream
        // beside the last forces
        cudaEventRecord(h->ev_rows, st);
        cudaStreamWaitEvent(s2, h->ev_rows, 0);
        k_degree_scatter<<<grid_for(n), kThreads, 0, s2>>>(d);
        cudaEventRecord(h->ev_join, s2);
      }
      k_row_fill<<<grid_for(std::max(b - a, 1)), kThreads, 0, st>>>(d, a, b);
      if (h->gcap > 0 || h->nfix > 0) k_force<true><<<h->num_sms * h->force_bps, kThreads, 0, st>>>(d, a, b);
      else k_force<false><<<h->num_sms * h->force_bps, kThreads, 0, st>>>(d, a, b);
    }
    cudaStreamWaitEvent(st, h->ev_join, 0);
  }
  mark(PH_GATHER);
  if (s2 == st) k_degree_scatter<<<grid_for(n), kThreads, 0, st>>>(d);
  k_gather<<<grid_for(n), kThreads, 0, st>>>(d);
  k_integrate<<<grid_for(n), kThreads, 0, st>>>(d);
  mark(PH_DELETE);
  k_finish<<<1, kThreads, 0, st>>>(d, h->scal + S_COUNTERS, h->scal, h->d_mirror, S_SIZE);
  mark(PH_END);
  h->mirror_ok = true;
  mark(kPhases);
  // bin, scan, scatter, cellorder, wall detect, wall force, degree scatter,
  // gather, integrate, finish; per chunk search, scan (3), row fill, force
  L += 1 + 3 + 1 + 1 + 1 + 1 + 3 + 1 + 6 * nchunk;
  h->launches += L;
  if (ev) h->prof_steps++;
  h->cur = 1 - h->cur;
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return cuda_fail(h, e, "kernel launch");
  return 0;
}

void drop_graph(sdem_h* h) {
  h->graph_gen++;
  if (h->graph2) cudaGraphExecDestroy(h->graph2);
  h->graph2 = nullptr;
  h->graph_cur = -1;
  for (int b = 0; b < 2; b++) {
    if (h->graph1[b]) cudaGraphExecDestroy(h->graph1[b]);
    h->graph1[b] = nullptr;
  }
}

// Reads the device scalars as of iteration `it` from its mirror slot (after
// that step completed), or the device copy when the mirror does not hold it.
int read_scalars(sdem_h* h, long long it, int* s) {
  const int* m = h->h_mirror + (it & 1) * S_SIZE;
  if (h->mirror_ok && m[S_ITER] == (int)it) std::memcpy(s, m, sizeof(int) * S_SIZE);
  else CK(cudaMemcpy(s, h->scal, sizeof(int) * S_SIZE, cudaMemcpyDeviceToHost));
  return 0;
}

int check_scalars(sdem_h* h, const int* s);

int sync_and_check(sdem_h* h) {
  CK(cudaStreamSynchronize(h->stream));
  int s[S_SIZE];
  int rc = read_scalars(h, h->iter_host, s);
  if (rc) return rc;
  return check_scalars(h, s);
}

// Takes the counters and the error status of a scalar snapshot.
int check_scalars(sdem_h* h, const int* s) {
  std::memcpy(h->h_counters, s + S_COUNTERS, sizeof(int) * SDEM_CNT_SIZE);
  if (s[S_STATUS] != 0) {
    int code = s[S_STATUS], detail = s[S_STATUS + 1];
    std::string msg;
    switch (code) {
      case SDEM_E_GRID: msg = "particle index " + std::to_string(detail) + " is outside the padded search grid"; break;
      case SDEM_E_CL_FULL: msg = "contact capacity exceeded (detail " + std::to_string(detail) +
                                 "): raise cntct_list_size or max_contacts_per_particle"; break;
      case SDEM_E_CAPACITY: msg = "too many out-of-domain particles in one step"; break;
      default: msg = "device error " + std::to_string(code) + " detail " + std::to_string(detail);
    }
    // clear so the handle stays usable for downloads
    int z[2] = {0, 0};
    cudaStreamSynchronize(h->stream);
    cudaMemcpyAsync(h->scal + S_STATUS, z, sizeof z, cudaMemcpyHostToDevice, h->stream);
    cudaStreamSynchronize(h->stream);
    h->mirror_ok = false;
    return set_err(h, code, msg);
  }
  return 0;
}

}  // namespace

// Message of the last failed sdem_count_contacts_noalloc on this thread
// (sdem_last_error(NULL) returns it).
namespace {
thread_local char g_noalloc_msg[160] = "";
}  // namespace

// ===========================================================================
extern "C" {

void sdem_default_cfg(sdem_cfg* c) {
  std::memset(c, 0, sizeof *c);
  c->n_capacity = 8000;
  c->max_gid = 8000;
  c->tsize = 1;
  c->rsize = 1;
  c->cf_type = SDEM_CFT_LSD;
  c->ct_model = SDEM_CTM_CONSTANT;
  c->pi_method = SDEM_PIM_FE;
  c->pri_method = SDEM_PIM_FE;
  c->cs_method = SDEM_CSM_NBS_MUNJIZA;
  c->cntct_list_size = 6;
  c->base_wall_id = 10000000;
  c->wall_max_update_iter = 100;
  c->quirk_ab2_rot = 1;
  c->max_contacts_per_particle = 0;
  c->dt = 1.0E-5;
  c->gravity[1] = -9.81;
  c->cs_ratio = 1.0;
  c->wall_neighbor_ratio = 2.0;
}

int sdem_create(const sdem_cfg* cfg, sdem_h** out) {
  if (!cfg || !out) return SDEM_E_ARG;
  *out = nullptr;
  sdem_h* h = new sdem_h();
  h->cfg = *cfg;
  const sdem_cfg& c = h->cfg;
  auto bad = [&](const char* m) {
    h->err = m;
    *out = h;
    return SDEM_E_ARG;
  };
  if (c.n_capacity < 1) return bad("n_capacity must be >= 1");
  if (c.max_gid < 1) return bad("max_gid must be >= 1");
  if (c.tsize < 1 || c.tsize > 3 || c.rsize < 1 || c.rsize > 3) return bad("tsize/rsize must be 1..3");
  if (c.pi_method < SDEM_PIM_FE || c.pi_method > SDEM_PIM_AB3 || c.pri_method < SDEM_PIM_FE ||
      c.pri_method > SDEM_PIM_AB3)
    return bad("PI_Method and PRI_Method must be 1 (FE), 2 (AB2) or 3 (AB3)");
  if (c.tsize < c.pi_method || c.rsize < c.pri_method) return bad("tsize >= PI_Method and rsize >= PRI_Method required");
  if (c.cf_type != SDEM_CFT_LSD && c.cf_type != SDEM_CFT_NLIN) return bad("cf_type must be 1 (LSD) or 2 (Hertz)");
  if (c.ct_model != SDEM_CTM_CONSTANT && c.ct_model != SDEM_CTM_VARIABLE) return bad("ct_model must be 1 or 2");
  if (c.cs_method != SDEM_CSM_NBS_MUNJIZA && c.cs_method != SDEM_CSM_HRCHL) return bad("cs_method must be 1 or 2");
  if (c.cs_method == SDEM_CSM_HRCHL && c.n_fixed_capacity > 0) {
    // NBSMH_LoopNBSMask has no fixed-particle branch (Prtcl_Hrchl_Munjiza.f90:601-704)
    h->err = "fixed spheres with the hierarchical search (CS_Method=2) are not supported";
    *out = h;
    return SDEM_E_UNSUPPORTED;
  }
  if (c.cs_num_levels < 0 || c.cs_num_levels > kMaxLevels) return bad("cs_num_levels must be 0..6");
  h->hier = c.cs_method == SDEM_CSM_HRCHL;
  if (c.max_gid >= kImgFlag) return bad("max_gid must be < 2^30");
  if (!(c.cs_ratio >= 1.0)) return bad("Prtcl_cs_ratio must be >= 1 for the one-level NBS search");
  const int nper = (c.periodic[0] != 0) + (c.periodic[1] != 0) + (c.periodic[2] != 0);
  // search positions pack into 26 bits; each periodic direction at most
  // doubles the particles the search sees (locals + images)
  if (((long long)c.n_capacity << nper) >= (1LL << 26)) return bad("n_capacity * 2^(periodic directions) must be < 2^26");
  if ((long long)std::max(1, c.cntct_list_size) * c.n_capacity >= (1ll << 30))
    return bad("cntct_list_size * n_capacity must be < 2^30");
  h->K = c.max_contacts_per_particle > 0 ? c.max_contacts_per_particle : 24;
  if (h->K > kMaxK) return bad("max_contacts_per_particle must be <= 64");
  *out = h;
  if (cudaGetDevice(&h->dev) != cudaSuccess) return set_err(h, SDEM_E_CUDA, "no CUDA device");
  CK(cudaDeviceGetAttribute(&h->num_sms, cudaDevAttrMultiProcessorCount, h->dev));
  CK(cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking));
  CK(cudaStreamCreateWithFlags(&h->stream2, cudaStreamNonBlocking));
  CK(cudaStreamCreateWithFlags(&h->stream_io, cudaStreamNonBlocking));
  CK(cudaEventCreateWithFlags(&h->ev_snap, cudaEventDisableTiming));
  CK(cudaEventCreateWithFlags(&h->ev_snap_done, cudaEventDisableTiming));
  CK(cudaEventCreateWithFlags(&h->ev_fork, cudaEventDisableTiming));
  CK(cudaEventCreateWithFlags(&h->ev_join, cudaEventDisableTiming));
  CK(cudaEventCreateWithFlags(&h->ev_rows, cudaEventDisableTiming));
  for (int k = 0; k < 6; k++) CK(cudaEventCreateWithFlags(&h->ev_xfer[k], cudaEventDisableTiming));
  for (int k = 0; k < kMaxChunks; k++) CK(cudaEventCreateWithFlags(&h->ev_chunk[k], cudaEventDisableTiming));
  int N = c.n_capacity;
  if (c.n_fixed_capacity < 0) return bad("n_fixed_capacity must be >= 0");
  if (c.n_fixed_capacity > 0 && nper > 0) {
    h->err = "fixed spheres with periodic directions are not implemented on the GPU";
    *out = h;
    return SDEM_E_UNSUPPORTED;
  }
  h->fcap = c.n_fixed_capacity;
  // Periodic images need room beside the particles in the search arrays.  A
  // periodic side longer than two search cells gives every point at most one
  // image per direction (the bands at both faces are disjoint), so the
  // points after the y, x and z passes number at most 2^(directions) per particle.
  h->gcap = (int)(((long long)N << nper) - N);
  if ((long long)N + h->gcap + h->fcap >= (1LL << 26))
    return bad("particles + periodic images + fixed spheres must stay below 2^26");
  const int NA = N + h->gcap + h->fcap;   // + fixed spheres after the images
  h->nall = NA;
  int rc = 0;
  rc |= dalloc(h, &h->gid, NA);
  rc |= dalloc(h, &h->ptype, NA);
  rc |= dalloc(h, &h->usrmark, N);
  rc |= dalloc(h, &h->posr, NA);
  for (int k = 0; k < 3; k++) {
    if (k < c.tsize) { rc |= dalloc(h, &h->vel[k], k == 0 ? NA : N); rc |= dalloc(h, &h->acc[k], N); }
    if (k < c.rsize) { rc |= dalloc(h, &h->rv[k], k == 0 ? NA : N); rc |= dalloc(h, &h->ra[k], N); }
  }
  if (h->gcap > 0) {
    rc |= dalloc(h, &h->gflag, (size_t)NA);
    rc |= dalloc(h, &h->goff, (size_t)NA + 1);
  }
  if (h->fcap > 0) {
    rc |= dalloc(h, &h->fix_gid, (size_t)h->fcap);
    rc |= dalloc(h, &h->fix_ptype, (size_t)h->fcap);
    rc |= dalloc(h, &h->fix_posr, (size_t)h->fcap);
  }
  rc |= dalloc(h, &h->theta, N);
  rc |= dalloc(h, &h->F, N);
  rc |= dalloc(h, &h->T, N);
  rc |= dalloc(h, &h->near_mask, N);
  rc |= dalloc(h, &h->cell_of, NA);
  rc |= dalloc(h, &h->tmp_rank, NA);
  rc |= dalloc(h, &h->tmp_sorted, NA);
  rc |= dalloc(h, &h->sorted, NA);
  rc |= dalloc(h, &h->sortpos, NA);
  rc |= dalloc(h, &h->spos, NA);
  rc |= dalloc(h, &h->pf, NA);
  rc |= dalloc(h, &h->pcell, NA);
  rc |= dalloc(h, &h->deg_cnt, kDegBuckets);
  rc |= dalloc(h, &h->deg_of, N);
  rc |= dalloc(h, &h->deg_rank, N);
  rc |= dalloc(h, &h->gorder, N);
  rc |= dalloc(h, &h->w_cnt, N);
  rc |= dalloc(h, &h->w_wall, (size_t)N * kKw);
  rc |= dalloc(h, &h->wl, (size_t)N * kKw);
  rc |= dalloc(h, &h->w_geo, (size_t)N * kKw);
  rc |= dalloc(h, &h->w_S, (size_t)N * kKw);
  rc |= dalloc(h, &h->w_M, (size_t)N * kKw);
  rc |= dalloc(h, &h->w_Mr, (size_t)N * kKw);
  rc |= dalloc(h, &h->row_cnt, NA);
  rc |= dalloc(h, &h->row_off, (size_t)NA + 1);
  rc |= dalloc(h, &h->row_partner, (size_t)NA * h->K);
  rc |= dalloc(h, &h->in_cnt, N);
  rc |= dalloc(h, &h->in_list, (size_t)N * h->K);
  h->ccap = std::max(1, c.cntct_list_size) * N;
  rc |= dalloc(h, &h->c_ogid, h->ccap);
  rc |= dalloc(h, &h->c_row, h->ccap);
  rc |= dalloc(h, &h->c_rec, h->ccap);
  size_t G = (size_t)c.max_gid + 1;
  for (int b = 0; b < 2; b++) {
    rc |= dalloc(h, &h->c_pgid[b], h->ccap);
    rc |= dalloc(h, &h->c_hist[b], h->ccap);
    rc |= dalloc(h, &h->own_cnt[b], G);
    rc |= dalloc(h, &h->own_c[b], G * h->K);
    rc |= dalloc(h, &h->wh_cnt[b], G);
    rc |= dalloc(h, &h->wh_wall[b], G * kKw);
    rc |= dalloc(h, &h->wh_hist[b], G * kKw);
  }
  rc |= dalloc(h, &h->scal, S_SIZE);
  rc |= dalloc(h, &h->ull, 10);
  rc |= dalloc(h, &h->red_part, 2 * (size_t)h->num_sms * kBeginBlocksPerSM);
  rc |= dalloc(h, &h->out_list, kOutCap);
  rc |= dalloc(h, &h->moves, 1 + 2 * 5 * kOutCap + 5 * kOutCap);
  rc |= dalloc(h, &h->map_pos, 5 * kOutCap);
  rc |= dalloc(h, &h->map_id, 5 * kOutCap);
  rc |= dalloc(h, &h->scan_tmp, 65536);
  if (rc) return SDEM_E_NOMEM;
  CK(cudaMallocHost(&h->h_counters, sizeof(int) * SDEM_CNT_SIZE));
  CK(cudaHostAlloc((void**)&h->h_mirror, sizeof(int) * 2 * S_SIZE, cudaHostAllocMapped));
  CK(cudaHostAlloc((void**)&h->h_chk, sizeof(int) * 2, cudaHostAllocDefault));
  std::memset(h->h_mirror, 0, sizeof(int) * 2 * S_SIZE);
  for (int b = 0; b < 2; b++) CK(cudaEventCreateWithFlags(&h->ev_step[b], cudaEventDisableTiming));
  CK(cudaHostGetDevicePointer((void**)&h->d_mirror, h->h_mirror, 0));
  std::memset(h->h_counters, 0, sizeof(int) * SDEM_CNT_SIZE);
  CK(cudaStreamSynchronize(h->stream));
  return 0;
}

int sdem_set_types(sdem_h* h, int nT, const double* radius, const double* mass, const double* inertia,
                   const double* bnry_pp, int nWT, const double* bnry_pw) {
  if (!h) return SDEM_E_ARG;
  if (nT < 1 || nWT < 1 || !radius || !mass || !inertia || !bnry_pp || !bnry_pw)
    return set_err(h, SDEM_E_ARG, "sdem_set_types: bad arguments");
  if (h->have_types) return set_err(h, SDEM_E_ARG, "sdem_set_types: tables are set once per handle");
  h->nT = nT;
  h->nWT = nWT;
  h->h_radius.assign(radius, radius + nT);
  int rc = 0;
  rc |= dalloc(h, &h->radius, nT);
  rc |= dalloc(h, &h->mass, nT);
  rc |= dalloc(h, &h->inertia, nT);
  rc |= dalloc(h, &h->bpp, (size_t)nT * nT * SDEM_BP_SIZE);
  rc |= dalloc(h, &h->bpw, (size_t)nT * nWT * SDEM_BP_SIZE);
  if (rc) return SDEM_E_NOMEM;
  CK(cudaMemcpyAsync(h->radius, radius, sizeof(double) * nT, cudaMemcpyHostToDevice, h->stream));
  CK(cudaMemcpyAsync(h->mass, mass, sizeof(double) * nT, cudaMemcpyHostToDevice, h->stream));
  CK(cudaMemcpyAsync(h->inertia, inertia, sizeof(double) * nT, cudaMemcpyHostToDevice, h->stream));
  CK(cudaMemcpyAsync(h->bpp, bnry_pp, sizeof(double) * nT * nT * SDEM_BP_SIZE, cudaMemcpyHostToDevice, h->stream));
  CK(cudaMemcpyAsync(h->bpw, bnry_pw, sizeof(double) * nT * nWT * SDEM_BP_SIZE, cudaMemcpyHostToDevice, h->stream));
  CK(cudaStreamSynchronize(h->stream));
  // Init_NBSM, Prtcl_NBS_Munjiza.f90:66-77 (one rank: subdomain = domain)
  double maxR = radius[0];
  for (int t = 1; t < nT; t++) maxR = std::max(maxR, radius[t]);
  h->maxR = maxR;
  const sdem_cfg& c = h->cfg;
  double maxDiam = 2.0 * maxR;
  h->cell = c.cs_ratio * maxDiam;
  h->x0 = c.dom_min[0] - h->cell * 1.05;
  h->y0 = c.dom_min[1] - h->cell * 1.05;
  h->z0 = c.dom_min[2] - h->cell * 1.05;
  double xed = c.dom_max[0] + h->cell * 1.05, yed = c.dom_max[1] + h->cell * 1.05, zed = c.dom_max[2] + h->cell * 1.05;
  h->nx = (int)((xed - h->x0) / h->cell) + 1;
  h->ny = (int)((yed - h->y0) / h->cell) + 1;
  h->nz = (int)((zed - h->z0) / h->cell) + 1;
  h->ncell = (long long)h->nx * h->ny * h->nz;
  if (h->hier) {
    // Init_Munjiza_Hrchl (Prtcl_Hrchl_Munjiza.f90:78-218): levels halve the
    // diameter bracket and the cell; every type of the table counts as
    // populated (an empty level finds nothing either way).  Levels here are
    // ordered coarsest first; the cell arrays hold the finest level first.
    double maxD = 0.0, minD = 0.0;
    for (int t = 0; t < nT; t++) {
      const double dd = 2.0 * radius[t];
      if (t == 0 || dd > maxD) maxD = dd;
      if (t == 0 || dd < minD) minD = dd;
    }
    const int dmax_min = (int)(maxD / minD);
    int numLevels = c.cs_num_levels > 0 ? c.cs_num_levels
                  : dmax_min <= 1 ? 1 : dmax_min <= 3 ? 2 : dmax_min <= 7 ? 3 : dmax_min <= 15 ? 4
                  : dmax_min <= 31 ? 5 : 6;
    std::vector<int> tl(nT, 0);
    h->nlvl = 0;
    double maxD_lvl = maxD, cl = h->cell;
    int nx = h->nx, ny = h->ny, nz = h->nz;
    for (int idh = 1; idh <= numLevels; idh++) {
      double minD_lvl = maxD_lvl / 2.0;
      if (idh == numLevels) minD_lvl = 0.0;
      bool populated = false;
      for (int t = 0; t < nT; t++) {
        const double dd = 2.0 * radius[t];
        if (dd > minD_lvl && (idh == 1 || dd <= maxD_lvl)) {
          populated = true;
          tl[t] = h->nlvl;
        }
      }
      if (populated) {
        LevelGrid& G = h->lv[h->nlvl++];
        G.nx = nx; G.ny = ny; G.nz = nz;
        G.mult = idh;
        G.cell = cl;
        G.cellf = (float)cl;
        G.div = fpi::divisor(cl);
      }
      nx *= 2; ny *= 2; nz *= 2;
      maxD_lvl = minD_lvl;
      cl = cl / 2.0;
    }
    long long off = 0;
    for (int k = h->nlvl - 1; k >= 0; k--) {
      h->lv[k].base = off;
      off += (long long)h->lv[k].nx * h->lv[k].ny * h->lv[k].nz;
    }
    h->ncell = off;
    rc |= dalloc(h, &h->type_lvl, (size_t)nT);
    if (rc) return SDEM_E_NOMEM;
    CK(cudaMemcpyAsync(h->type_lvl, tl.data(), sizeof(int) * nT, cudaMemcpyHostToDevice, h->stream));
    CK(cudaStreamSynchronize(h->stream));
  }
  {
    double mn = std::min(c.dom_max[0] - c.dom_min[0], std::min(c.dom_max[1] - c.dom_min[1], c.dom_max[2] - c.dom_min[2]));
    if (1.02 * h->cell > mn) return set_err(h, SDEM_E_ARG, "PC_InitComm: so big Diameter (domain narrower than 1.02 cells)");
    for (int k = 0; k < 3; k++)
      if (c.periodic[k] && !(c.dom_max[k] - c.dom_min[k] > 2.0 * h->cell))
        return set_err(h, SDEM_E_UNSUPPORTED, "a periodic side must be longer than two search cells on the GPU");
  }
  // Single-precision prefilter of the search: coordinates are stored relative to
  // their cell corner (|value| < 1 cell), so each rounding (coordinate, radius,
  // cell size, differences, squares and sums) is below cell*2^-23; their sum
  // bounds the distance error by ~8*cell*2^-23, and the margin is four times
  // that.
  h->pf_margin = (float)(32.0 * h->cell * std::ldexp(1.0, -23));
  if (h->ncell >= (1ll << 31) - 1) return set_err(h, SDEM_E_ARG, "search grid has more than 2^31 cells");
  rc |= dalloc(h, &h->cell_cnt, (size_t)h->ncell);
  rc |= dalloc(h, &h->cell_start, (size_t)h->ncell + 1);
  if (rc) return SDEM_E_NOMEM;
  long long nb = std::max<long long>((h->ncell + kScanTile - 1) / kScanTile, ((long long)h->nall + kScanTile - 1) / kScanTile);
  if (nb > 65536) {
    rc |= dalloc(h, &h->scan_tmp, (size_t)nb);
    if (rc) return SDEM_E_NOMEM;
  }
  CK(cudaStreamSynchronize(h->stream));
  h->have_types = true;
  return 0;
}

int sdem_set_walls(sdem_h* h, int nw, const double* wall, const int* flags) {
  if (!h) return SDEM_E_ARG;
  if (nw < 0 || nw > kMaxWalls) return set_err(h, SDEM_E_ARG, "sdem_set_walls: 0 <= nw <= 64");
  if (nw > 0 && (!wall || !flags)) return set_err(h, SDEM_E_ARG, "sdem_set_walls: null arrays");
  h->nw = nw;
  h->h_wall_id.assign(nw, 0);
  double mv = 0.0;
  for (int k = 0; k < nw; k++) {
    const double* v = wall + (size_t)k * SDEM_W_SIZE + SDEM_W_VEL;
    double s = std::sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
    mv = (mv > s) ? mv : s;
    h->h_wall_id[k] = flags[(size_t)k * SDEM_WF_SIZE + SDEM_WF_WALL_ID];
    int wt = flags[(size_t)k * SDEM_WF_SIZE + SDEM_WF_WALL_TYPE];
    if (h->have_types && (wt < 1 || wt > h->nWT)) return set_err(h, SDEM_E_ARG, "sdem_set_walls: wall_Type out of range");
  }
  h->max_wall_vel = mv;
  int rc = 0;
  if (!h->walls) {
    rc |= dalloc(h, &h->walls, (size_t)kMaxWalls * SDEM_W_SIZE);
    rc |= dalloc(h, &h->wflags, (size_t)kMaxWalls * SDEM_WF_SIZE);
    if (rc) return SDEM_E_NOMEM;
  }
  if (nw > 0) {
    CK(cudaMemcpyAsync(h->walls, wall, sizeof(double) * nw * SDEM_W_SIZE, cudaMemcpyHostToDevice, h->stream));
    CK(cudaMemcpyAsync(h->wflags, flags, sizeof(int) * nw * SDEM_WF_SIZE, cudaMemcpyHostToDevice, h->stream));
  }
  drop_graph(h);
  // the near-wall list is rebuilt at the next step
  int zero = 0;
  CK(cudaMemcpyAsync(h->scal + S_NEXT, &zero, sizeof zero, cudaMemcpyHostToDevice, h->stream));
  h->mirror_ok = false;
  CK(cudaStreamSynchronize(h->stream));
  return 0;
}

int sdem_set_fixed(sdem_h* h, int nfix, const int* id, const int* ptype, const double* pos) {
  if (!h) return SDEM_E_ARG;
  const sdem_cfg& c = h->cfg;
  if (!h->have_types) return set_err(h, SDEM_E_ARG, "sdem_set_fixed: call sdem_set_types first");
  if (nfix < 0 || (nfix > 0 && (!id || !ptype || !pos))) return set_err(h, SDEM_E_ARG, "sdem_set_fixed: bad arguments");
  if (nfix > h->fcap) return set_err(h, SDEM_E_CAPACITY, "sdem_set_fixed: more fixed spheres than n_fixed_capacity");
  std::vector<int> g, t;
  std::vector<dbl4> p;
  for (int i = 0; i < nfix; i++) {
    if (ptype[i] < 1 || ptype[i] > h->nT) return set_err(h, SDEM_E_ARG, "sdem_set_fixed: type outside 1..nT");
    if (id[i] <= c.max_gid || id[i] >= c.base_wall_id)
      return set_err(h, SDEM_E_BAD_ID, "sdem_set_fixed: fixed ids must lie above max_gid and below base_wall_id");
    const double x = pos[3 * i], y = pos[3 * i + 1], z = pos[3 * i + 2];
    // PIO_ReadFixedCoord keeps the spheres of this rank's subdomain (:222)
    if (!(x >= c.dom_min[0] && x < c.dom_max[0] && y >= c.dom_min[1] && y < c.dom_max[1] && z >= c.dom_min[2] &&
          z < c.dom_max[2]))
      continue;
    g.push_back(id[i]);
    t.push_back(ptype[i]);
    p.push_back(make_dbl4(x, y, z, h->h_radius[ptype[i] - 1]));
  }
  CK(cudaStreamSynchronize(h->stream));
  if (!g.empty()) {
    CK(cudaMemcpyAsync(h->fix_gid, g.data(), sizeof(int) * g.size(), cudaMemcpyHostToDevice, h->stream));
    CK(cudaMemcpyAsync(h->fix_ptype, t.data(), sizeof(int) * t.size(), cudaMemcpyHostToDevice, h->stream));
    CK(cudaMemcpyAsync(h->fix_posr, p.data(), sizeof(dbl4) * p.size(), cudaMemcpyHostToDevice, h->stream));
  }
  CK(cudaStreamSynchronize(h->stream));
  h->nfix = (int)g.size();
  drop_graph(h);   // the step graph bakes in the search length
  return 0;
}

int sdem_upload_particles(sdem_h* h, int n, const int* id, const int* ptype, const int* usrmark, const double* posR,
                          const double* linVel, const double* linAcc, const double* theta, const double* rotVel,
                          const double* rotAcc) {
  if (!h) return SDEM_E_ARG;
  const sdem_cfg& c = h->cfg;
  if (!h->have_types) return set_err(h, SDEM_E_ARG, "sdem_upload_particles: call sdem_set_types first");
  if (n < 0 || n > c.n_capacity) return set_err(h, SDEM_E_CAPACITY, "sdem_upload_particles: n exceeds n_capacity");
  if (n > 0 && (!id || !ptype || !posR || !linVel)) return set_err(h, SDEM_E_ARG, "sdem_upload_particles: null arrays");
  // Stream-ordered copies: a step still in flight finishes before the state
  // is replaced, and the call returns after the last copy has landed.  The
  // copies follow one another on the handle's stream; each staged field is
  // unpacked on the second stream once its copy has landed, beside the next
  // copy.  The device's check of ids and types is read back at the end.
  cudaStream_t st = h->stream, s2 = h->stream2;
  CK(cudaStreamSynchronize(st));
  h->mirror_ok = false;   // the device scalars are rewritten below
  int chk[2] = {0, 0};
  int* scal = h->scal;
  if (n > 0) {
    CK(cudaMemcpyAsync(h->gid, id, sizeof(int) * n, cudaMemcpyHostToDevice, st));
    CK(cudaMemcpyAsync(h->ptype, ptype, sizeof(int) * n, cudaMemcpyHostToDevice, st));
    // ids and types are checked on the device (the owner table of buffer 0,
    // cleared again below, holds the per-id flags)
    CK(cudaMemsetAsync(h->own_cnt[0], 0, sizeof(int) * ((size_t)c.max_gid + 1), st));
    CK(cudaMemsetAsync(scal + S_STATUS, 0, 2 * sizeof(int), st));
    k_check_upload<<<grid_for(n), kThreads, 0, st>>>(h->gid, h->ptype, n, c.max_gid, h->nT, h->own_cnt[0],
                                                     scal + S_STATUS);
    CK(cudaMemcpyAsync(h->h_chk, scal + S_STATUS, 2 * sizeof(int), cudaMemcpyDeviceToHost, st));
    if (usrmark) CK(cudaMemcpyAsync(h->usrmark, usrmark, sizeof(int) * n, cudaMemcpyHostToDevice, st));
    else CK(cudaMemsetAsync(h->usrmark, 0, sizeof(int) * n, st));
    // (x, y, z, r) per particle is also the device record
    CK(cudaMemcpyAsync(h->posr, posR, sizeof(dbl4) * n, cudaMemcpyHostToDevice, st));
    const size_t per = 3 * (size_t)(2 * c.tsize + 2 * c.rsize + 1);
    int rs = ensure_stage(h, per * n);
    if (rs) return rs;
    double* sp = h->stage;
    int f = 0;
    auto put = [&](const double* src, int levels, dbl4* const* dst) {
      if (src) CK(cudaMemcpyAsync(sp, src, sizeof(double) * 3 * levels * (size_t)n, cudaMemcpyHostToDevice, st));
      CK(cudaEventRecord(h->ev_xfer[f], st));
      CK(cudaStreamWaitEvent(s2, h->ev_xfer[f], 0));
      for (int k = 0; k < levels; k++) k_unpack3<<<grid_for(n), kThreads, 0, s2>>>(dst[k], src ? sp : nullptr, n, levels, k);
      sp += 3 * (size_t)levels * n;
      f++;
      return 0;
    };
    dbl4* th[1] = {h->theta};
    int rc = put(linVel, c.tsize, h->vel);
    rc |= put(linAcc, c.tsize, h->acc);
    rc |= put(theta, 1, th);
    rc |= put(rotVel, c.rsize, h->rv);
    rc |= put(rotAcc, c.rsize, h->ra);
    if (rc) return rc;
    CK(cudaEventRecord(h->ev_xfer[5], s2));
    CK(cudaStreamWaitEvent(st, h->ev_xfer[5], 0));
    k_tag_vel<<<grid_for(n), kThreads, 0, st>>>(h->vel[0], h->gid, h->ptype, n);
  }
  // history reset: both buffers empty; near-wall list refreshed at the next step
  size_t G = (size_t)c.max_gid + 1;
  for (int b = 0; b < 2; b++) {
    CK(cudaMemsetAsync(h->own_cnt[b], 0, sizeof(int) * G, st));
    CK(cudaMemsetAsync(h->wh_cnt[b], 0, sizeof(int) * G, st));
  }
  h->h_up.clear();
  CK(cudaMemsetAsync(h->F, 0, sizeof(dbl4) * c.n_capacity, st));
  CK(cudaMemsetAsync(h->T, 0, sizeof(dbl4) * c.n_capacity, st));
  CK(cudaMemsetAsync(h->near_mask, 0, sizeof(unsigned long long) * c.n_capacity, st));
  int sc[S_SIZE] = {0};
  sc[S_N] = n;
  sc[S_NT] = n;
  CK(cudaMemcpyAsync(h->scal, sc, sizeof sc, cudaMemcpyHostToDevice, st));
  CK(cudaMemsetAsync(h->ull, 0, sizeof(unsigned long long) * 10, st));
  CK(cudaGetLastError());
  CK(cudaStreamSynchronize(st));
  if (n > 0) std::memcpy(chk, h->h_chk, sizeof chk);
  if (chk[0] != 0) {
    h->n_host = 0;   // the handle holds no valid particle set now
    h->stepped = false;
    drop_graph(h);
    const int zs[S_SIZE] = {0};   // no particles, status cleared
    CK(cudaMemcpy(scal, zs, sizeof zs, cudaMemcpyHostToDevice));
    const std::string at = " (particle index " + std::to_string(chk[1]) + ")";
    if (chk[0] == SDEM_E_BAD_ID) return set_err(h, SDEM_E_BAD_ID, "particle id outside 1..max_gid" + at);
    if (chk[0] == SDEM_E_BAD_ID + 100) return set_err(h, SDEM_E_BAD_ID, "duplicate particle id" + at);
    return set_err(h, SDEM_E_ARG, "particle type outside 1..nT" + at);
  }
  // the captured step graphs bake in launch sizes from the particle count
  // (and nothing else that an upload changes): they stay valid for a new
  // particle set of the same size
  if (n != h->n_host) drop_graph(h);
  h->n_host = n;
  h->cur = 0;
  h->stepped = false;
  // the iteration count restarts at 0: no mirror slot or step event may
  // stand for an iteration of the new run
  std::memset(h->h_mirror, 0, sizeof(int) * 2 * S_SIZE);
  h->iter_host = 0;
  h->ev_iter[0] = h->ev_iter[1] = -1;
  std::memset(h->h_counters, 0, sizeof(int) * SDEM_CNT_SIZE);
  h->h_counters[SDEM_CNT_NLOCAL] = n;
  return 0;
}

int sdem_upload_contacts(sdem_h* h, int nc, const int* owner_idx, const int* partner_id, const double* tandelta,
                         const double* velrel) {
  if (!h) return SDEM_E_ARG;
  if (nc < 0 || (nc > 0 && (!owner_idx || !partner_id || !tandelta || !velrel)))
    return set_err(h, SDEM_E_ARG, "sdem_upload_contacts: bad arguments");
  const sdem_cfg& c = h->cfg;
  int n = h->n_host;
  CK(cudaStreamSynchronize(h->stream));
  // The history the next step reads is the "previous" buffer.
  int pv = 1 - h->cur;
  std::vector<std::vector<std::pair<int, dbl4>>> wl(n);
  std::vector<sdem_h::UpRec> pp;
  std::vector<int> hg(std::max(n, 1));
  if (n > 0) CK(cudaMemcpy(hg.data(), h->gid, sizeof(int) * n, cudaMemcpyDeviceToHost));
  std::unordered_map<int, int> idx_of;
  for (int i = 0; i < n; i++) idx_of[hg[i]] = i;
  std::vector<double> posr(4 * (size_t)std::max(n, 1));
  if (n > 0) {
    std::vector<dbl4> pb(n);
    CK(cudaMemcpy(pb.data(), h->posr, sizeof(dbl4) * n, cudaMemcpyDeviceToHost));
    for (int i = 0; i < n; i++) {
      posr[4 * i] = pb[i].x; posr[4 * i + 1] = pb[i].y; posr[4 * i + 2] = pb[i].z; posr[4 * i + 3] = pb[i].w;
    }
  }
  for (int i = 0; i < nc; i++) {
    int o = owner_idx[i];
    if (o < 0 || o >= n) return set_err(h, SDEM_E_ARG, "sdem_upload_contacts: owner index out of range");
    int go = hg[o], pid = partner_id[i];
    dbl4 hist = make_dbl4(tandelta[3 * i], tandelta[3 * i + 1], tandelta[3 * i + 2], velrel[i]);
    if (pid > c.base_wall_id) {
      int wi = -1;
      for (int k = 0; k < h->nw; k++)
        if (h->h_wall_id[k] == pid) { wi = k; break; }
      if (wi < 0) continue;  // a wall this handle does not have: the record is never looked up
      bool dup = false;
      for (auto& e : wl[o]) dup |= (e.first == wi);
      if (!dup) wl[o].push_back({wi, hist});
      continue;
    }
    // CL_Add_RestartCntctlink (Prtcl_CL_and_CF.f90:577-622): a pair whose
    // partner is local and lies within 1.5*(r1+r2) is kept once, in the lower
    // id's bucket; any other record (a partner across a periodic boundary or
    // absent) stays in the owner's bucket
    bool both = false;
    auto it = idx_of.find(pid);
    if (it != idx_of.end()) {
      const double* a = &posr[4 * (size_t)o];
      const double* q = &posr[4 * (size_t)it->second];
      double dx = a[0] - q[0], dy = a[1] - q[1], dz = a[2] - q[2];
      double dist = std::sqrt(dx * dx + dy * dy + dz * dz) - 1.5 * (a[3] + q[3]);
      if (go > pid && dist <= 0.0) continue;
      both = (go < pid && dist <= 0.0);
    }
    pp.push_back({go, pid, both, hist});
  }
  // Find_insert walks a bucket from its newest record: of two records with
  // one key the later one is found
  std::stable_sort(pp.begin(), pp.end(), [](const sdem_h::UpRec& a, const sdem_h::UpRec& b) {
    return a.owner < b.owner || (a.owner == b.owner && a.partner < b.partner);
  });
  {
    std::vector<sdem_h::UpRec> u;
    for (size_t i = 0; i < pp.size(); i++)
      if (i + 1 == pp.size() || pp[i + 1].owner != pp[i].owner || pp[i + 1].partner != pp[i].partner) u.push_back(pp[i]);
    pp.swap(u);
  }
  if ((long long)pp.size() > h->ccap) return set_err(h, SDEM_E_CL_FULL, "sdem_upload_contacts: more records than contact capacity");
  size_t G = (size_t)c.max_gid + 1;
  std::vector<int> ocnt(G, 0), pg(pp.size());
  std::vector<int2> oc(G * h->K, make_int2(0, 0));
  std::vector<dbl4> hs(pp.size());
  for (size_t i = 0; i < pp.size(); i++) {
    int g = pp[i].owner;
    if (ocnt[g] >= h->K)
      return set_err(h, SDEM_E_CL_FULL, "sdem_upload_contacts: more records on one particle than max_contacts_per_particle");
    oc[(size_t)g * h->K + ocnt[g]++] = make_int2((int)i, pp[i].partner);
    pg[i] = pp[i].partner;
    hs[i] = pp[i].hist;
  }
  CK(cudaMemcpyAsync(h->own_cnt[pv], ocnt.data(), sizeof(int) * G, cudaMemcpyHostToDevice, h->stream));
  CK(cudaMemcpyAsync(h->own_c[pv], oc.data(), sizeof(int2) * G * h->K, cudaMemcpyHostToDevice, h->stream));
  if (!pp.empty()) {
    CK(cudaMemcpyAsync(h->c_pgid[pv], pg.data(), sizeof(int) * pp.size(), cudaMemcpyHostToDevice, h->stream));
    CK(cudaMemcpyAsync(h->c_hist[pv], hs.data(), sizeof(dbl4) * pp.size(), cudaMemcpyHostToDevice, h->stream));
  }
  h->h_up = pp;
  std::vector<int> whc(G, 0), whw(G * kKw, 0);
  std::vector<dbl4> whh(G * kKw);
  for (int o = 0; o < n; o++) {
    int g = hg[o];
    int k = 0;
    for (auto& e : wl[o]) {
      if (k >= kKw) return set_err(h, SDEM_E_CL_FULL, "sdem_upload_contacts: more than 4 wall contacts on one particle");
      whw[(size_t)g * kKw + k] = e.first;
      whh[(size_t)g * kKw + k] = e.second;
      k++;
    }
    whc[g] = k;
  }
  CK(cudaMemcpyAsync(h->wh_cnt[pv], whc.data(), sizeof(int) * G, cudaMemcpyHostToDevice, h->stream));
  CK(cudaMemcpyAsync(h->wh_wall[pv], whw.data(), sizeof(int) * G * kKw, cudaMemcpyHostToDevice, h->stream));
  CK(cudaMemcpyAsync(h->wh_hist[pv], whh.data(), sizeof(dbl4) * G * kKw, cudaMemcpyHostToDevice, h->stream));
  CK(cudaStreamSynchronize(h->stream));   // the host tables above go out of scope
  return 0;
}

namespace {
// Captures two steps into h->graph2 (starting from the current buffer parity).
int build_graph(sdem_h* h) {
  drop_graph(h);
  cudaGraph_t g = nullptr;
  int cur0 = h->cur;
  long long l0 = h->launches;
  CK(cudaStreamBeginCapture(h->stream, cudaStreamCaptureModeThreadLocal));
  int rc = enqueue_step(h);
  if (!rc) rc = enqueue_step(h);
  cudaError_t e = cudaStreamEndCapture(h->stream, &g);
  h->cur = cur0;  // capture does not execute; replays advance the parity
  h->graph_launches = h->launches - l0;
  h->launches = l0;
  if (rc) {
    if (g) cudaGraphDestroy(g);
    return rc;
  }
  if (e != cudaSuccess) return cuda_fail(h, e, "cudaStreamEndCapture");
  e = cudaGraphInstantiate(&h->graph2, g, 0);
  cudaGraphDestroy(g);
  if (e != cudaSuccess) {
    h->graph2 = nullptr;
    return cuda_fail(h, e, "cudaGraphInstantiate");
  }
  h->graph_cur = cur0;
  return 0;
}

// Captures one step starting from the current buffer parity into
// h->graph1[parity] (single steps, e.g. between output steps).
int build_graph1(sdem_h* h) {
  const int cur0 = h->cur;
  cudaGraph_t g = nullptr;
  long long l0 = h->launches;
  CK(cudaStreamBeginCapture(h->stream, cudaStreamCaptureModeThreadLocal));
  int rc = enqueue_step(h);
  cudaError_t e = cudaStreamEndCapture(h->stream, &g);
  h->cur = cur0;
  h->graph1_launches = h->launches - l0;
  h->launches = l0;
  if (rc) {
    if (g) cudaGraphDestroy(g);
    return rc;
  }
  if (e != cudaSuccess) return cuda_fail(h, e, "cudaStreamEndCapture");
  e = cudaGraphInstantiate(&h->graph1[cur0], g, 0);
  cudaGraphDestroy(g);
  if (e != cudaSuccess) {
    h->graph1[cur0] = nullptr;
    return cuda_fail(h, e, "cudaGraphInstantiate");
  }
  return 0;
}
}  // namespace

// Records the completion event of the step just enqueued (the one ending on
// iteration iter_host).
void mark_step(sdem_h* h) {
  h->mirror_ok = true;   // every step ends by copying the scalars to its mirror slot
  const int b = (int)(h->iter_host & 1);
  if (cudaEventRecord(h->ev_step[b], h->stream) == cudaSuccess) h->ev_iter[b] = h->iter_host;
  else h->ev_iter[b] = -1;
}

int sdem_step_async(sdem_h* h, int nsteps) {
  if (!h) return SDEM_E_ARG;
  if (!h->have_types) return set_err(h, SDEM_E_ARG, "sdem_step: call sdem_set_types first");
  if (nsteps < 0) return set_err(h, SDEM_E_ARG, "sdem_step: nsteps < 0");
  if (h->n_host == 0) return 0;
  int left = nsteps;
  // Long runs replay a captured two-step graph; profiling keeps plain launches
  // (its events differ per step).
  if (h->use_graphs && !h->prof && left >= 4) {
    if (h->graph2 == nullptr || h->graph_cur != h->cur) {
      if (h->graph2 && h->graph_cur != h->cur) {
        int rc = enqueue_step(h);  // realign the parity instead of capturing twice
        if (rc) return rc;
        left--;
        h->iter_host += 1;
        mark_step(h);
      }
      if (h->graph2 == nullptr) {
        int rc = build_graph(h);
        if (rc) return rc;
      }
    }
    while (left >= 2) {
      CK(cudaGraphLaunch(h->graph2, h->stream));
      h->launches += h->graph_launches;
      left -= 2;
      h->iter_host += 2;
      mark_step(h);
    }
  }
  for (int i = 0; i < left; i++) {
    if (h->use_graphs && !h->prof) {
      // a captured single step of this parity: one launch instead of ~25
      if (!h->graph1[h->cur]) {
        int rc = build_graph1(h);
        if (rc) return rc;
      }
      CK(cudaGraphLaunch(h->graph1[h->cur], h->stream));
      h->launches += h->graph1_launches;
      h->cur = 1 - h->cur;
    } else {
      int rc = enqueue_step(h);
      if (rc) return rc;
    }
    h->iter_host += 1;
    mark_step(h);
  }
  h->stepped = h->stepped || nsteps > 0;
  return 0;
}

int sdem_step(sdem_h* h, int nsteps) {
  int rc = sdem_step_async(h, nsteps);
  if (rc) return rc;
  return sync_and_check(h);
}

int sdem_get_stream(sdem_h* h, void** stream) {
  if (!h || !stream) return SDEM_E_ARG;
  *stream = (void*)h->stream;
  return 0;
}

int sdem_download_particles(sdem_h* h, int* n_out, int* id, int* ptype, int* usrmark, double* posR, double* linVel,
                            double* linAcc, double* theta, double* rotVel, double* rotAcc) {
  if (!h) return SDEM_E_ARG;
  int rc = sync_and_check(h);
  if (rc && rc != SDEM_E_CL_FULL && rc != SDEM_E_GRID && rc != SDEM_E_CAPACITY) return rc;
  int n = 0;
  CK(cudaMemcpy(&n, h->scal + S_N, sizeof n, cudaMemcpyDeviceToHost));
  if (n_out) *n_out = n;
  const sdem_cfg& c = h->cfg;
  cudaStream_t st = h->stream, s2 = h->stream2;
  if (n <= 0) return 0;
  const size_t per = 3 * (size_t)(2 * c.tsize + 2 * c.rsize + 1);
  rc = ensure_stage(h, per * n);
  if (rc) return rc;
  // The staged fields are packed on the second stream while the handle's
  // stream copies the records that need no packing; each staged field is
  // copied out once its packing is done, so the copies follow one another.
  CK(cudaEventRecord(h->ev_xfer[5], st));
  CK(cudaStreamWaitEvent(s2, h->ev_xfer[5], 0));
  struct Field {
    double* dst;
    int levels;
    dbl4* const* src;
  };
  dbl4* th[1] = {h->theta};
  const Field fs[5] = {{linVel, c.tsize, h->vel}, {linAcc, c.tsize, h->acc}, {theta, 1, th},
                       {rotVel, c.rsize, h->rv}, {rotAcc, c.rsize, h->ra}};
  double* sp = h->stage;
  for (int f = 0; f < 5; f++) {
    if (fs[f].dst)
      for (int k = 0; k < fs[f].levels; k++)
        k_pack3<<<grid_for(n), kThreads, 0, s2>>>(sp, fs[f].src[k], n, fs[f].levels, k);
    CK(cudaEventRecord(h->ev_xfer[f], s2));
    sp += 3 * (size_t)fs[f].levels * n;
  }
  if (id) CK(cudaMemcpyAsync(id, h->gid, sizeof(int) * n, cudaMemcpyDeviceToHost, st));
  if (ptype) CK(cudaMemcpyAsync(ptype, h->ptype, sizeof(int) * n, cudaMemcpyDeviceToHost, st));
  if (usrmark) CK(cudaMemcpyAsync(usrmark, h->usrmark, sizeof(int) * n, cudaMemcpyDeviceToHost, st));
  if (posR) CK(cudaMemcpyAsync(posR, h->posr, sizeof(dbl4) * n, cudaMemcpyDeviceToHost, st));
  sp = h->stage;
  for (int f = 0; f < 5; f++) {
    CK(cudaStreamWaitEvent(st, h->ev_xfer[f], 0));
    if (fs[f].dst)
      CK(cudaMemcpyAsync(fs[f].dst, sp, sizeof(double) * 3 * fs[f].levels * (size_t)n, cudaMemcpyDeviceToHost, st));
    sp += 3 * (size_t)fs[f].levels * n;
  }
  CK(cudaGetLastError());
  CK(cudaStreamSynchronize(st));
  return 0;
}

int sdem_download_forces(sdem_h* h, double* F, double* T) {
  if (!h) return SDEM_E_ARG;
  int rc = sync_and_check(h);
  if (rc) return rc;
  int n = 0;
  CK(cudaMemcpy(&n, h->scal + S_N, sizeof n, cudaMemcpyDeviceToHost));
  if (n <= 0) return 0;
  cudaStream_t st = h->stream;
  rc = ensure_stage(h, 6 * (size_t)n);
  if (rc) return rc;
  if (F) {
    k_pack3<<<grid_for(n), kThreads, 0, st>>>(h->stage, h->F, n, 1, 0);
    CK(cudaMemcpyAsync(F, h->stage, sizeof(double) * 3 * (size_t)n, cudaMemcpyDeviceToHost, st));
  }
  if (T) {
    k_pack3<<<grid_for(n), kThreads, 0, st>>>(h->stage + 3 * (size_t)n, h->T, n, 1, 0);
    CK(cudaMemcpyAsync(T, h->stage + 3 * (size_t)n, sizeof(double) * 3 * (size_t)n, cudaMemcpyDeviceToHost, st));
  }
  CK(cudaGetLastError());
  CK(cudaStreamSynchronize(st));
  return 0;
}

namespace {
struct CRec { int owner, partner; double t[3]; double vr; };

// Lays a contact snapshot for N particles and ccap records over `base`
// (32-byte aligned pieces); returns the bytes it needs.
size_t snap_layout(char* base, size_t N, size_t ccap, SnapContacts* sc) {
  size_t off = 0;
  auto take = [&](size_t bytes) {
    char* p = base ? base + off : nullptr;
    off += (bytes + 31) & ~(size_t)31;
    return p;
  };
  SnapContacts t;
  t.scal = (int*)take(2 * sizeof(int));
  t.gid = (int*)take(N * sizeof(int));
  t.og = (int*)take(ccap * sizeof(int));
  t.pg = (int*)take(ccap * sizeof(int));
  t.hs = (dbl4*)take(ccap * sizeof(dbl4));
  t.wcnt = (int*)take(N * sizeof(int));
  t.wwall = (int*)take(N * kKw * sizeof(int));
  t.whist = (dbl4*)take(N * kKw * sizeof(dbl4));
  if (sc) *sc = t;
  return off;
}

int ensure_snapshot_buffers(sdem_h* h, bool contacts) {
  const sdem_cfg& c = h->cfg;
  const size_t N = (size_t)c.n_capacity;
  if (!h->sn_state) {
    const size_t nd = N * (4 + 3 * (size_t)(2 * c.tsize + 2 * c.rsize + 1) + 6);
    cudaError_t e = cudaMalloc((void**)&h->sn_state, nd * sizeof(double));
    if (e == cudaSuccess) e = cudaMalloc((void**)&h->sn_ints, (3 * N + 1) * sizeof(int));
    if (e == cudaSuccess && !h->sn_n_host) e = cudaHostAlloc((void**)&h->sn_n_host, sizeof(int), cudaHostAllocDefault);
    if (e != cudaSuccess) {
      cudaGetLastError();
      return set_err(h, SDEM_E_NOMEM, "allocation of the output snapshot buffers failed");
    }
  }
  if (contacts && !h->sn_cdev) {
    const size_t bytes = snap_layout(nullptr, N, (size_t)h->ccap, nullptr);
    cudaError_t e = cudaMalloc(&h->sn_cdev, bytes);
    if (e == cudaSuccess) e = cudaHostAlloc(&h->sn_chost, bytes, cudaHostAllocMapped);
    void* hd = nullptr;
    if (e == cudaSuccess) e = cudaHostGetDevicePointer(&hd, h->sn_chost, 0);
    if (e != cudaSuccess) {
      cudaGetLastError();
      return set_err(h, SDEM_E_NOMEM, "allocation of the contact snapshot buffers failed");
    }
    snap_layout((char*)h->sn_cdev, N, (size_t)h->ccap, &h->sn_dev);
    snap_layout((char*)h->sn_chost, N, (size_t)h->ccap, &h->sn_host);
    snap_layout((char*)hd, N, (size_t)h->ccap, &h->sn_host_dptr);
  }
  return 0;
}

// Enqueues a snapshot: the frozen copy on the main stream (after every step
// enqueued so far), its download on the I/O stream.  Null host pointers are
// skipped.
int snapshot_begin(sdem_h* h, int* id, int* ptype, int* usrmark, double* posR, double* linVel, double* linAcc,
                   double* theta, double* rotVel, double* rotAcc, double* F, double* T, bool contacts) {
  if (h->snap_busy) {
    CK(cudaEventSynchronize(h->ev_snap_done));
    h->snap_busy = false;
  }
  int rc = ensure_snapshot_buffers(h, contacts);
  if (rc) return rc;
  const sdem_cfg& c = h->cfg;
  const int n = h->n_host;   // rows copied: the device count never exceeds it
  const size_t N = (size_t)c.n_capacity;
  cudaStream_t st = h->stream, io = h->stream_io;
  int* s_id = h->sn_ints;
  int* s_pt = s_id + N;
  int* s_um = s_pt + N;
  int* s_n = s_um + N;
  double* s_pos = h->sn_state;
  double* s_vec = s_pos + 4 * N;
  CK(cudaMemcpyAsync(s_n, h->scal + S_N, sizeof(int), cudaMemcpyDeviceToDevice, st));
  if (n > 0) {
    if (id) CK(cudaMemcpyAsync(s_id, h->gid, sizeof(int) * n, cudaMemcpyDeviceToDevice, st));
    if (ptype) CK(cudaMemcpyAsync(s_pt, h->ptype, sizeof(int) * n, cudaMemcpyDeviceToDevice, st));
    if (usrmark) CK(cudaMemcpyAsync(s_um, h->usrmark, sizeof(int) * n, cudaMemcpyDeviceToDevice, st));
    if (posR) CK(cudaMemcpyAsync(s_pos, h->posr, sizeof(dbl4) * n, cudaMemcpyDeviceToDevice, st));
  }
  // 3-vector fields in their host layouts, one after another
  struct Field { double* host; int levels; dbl4* const* dev; };
  dbl4* th[1] = {h->theta};
  dbl4* fF[1] = {h->F};
  dbl4* fT[1] = {h->T};
  const Field fields[7] = {{linVel, c.tsize, h->vel}, {linAcc, c.tsize, h->acc}, {theta, 1, th},
                           {rotVel, c.rsize, h->rv}, {rotAcc, c.rsize, h->ra}, {F, 1, fF}, {T, 1, fT}};
  double* sp = s_vec;
  double* where[7];
  for (int f = 0; f < 7; f++) {
    where[f] = sp;
    if (fields[f].host && n > 0)
      for (int k = 0; k < fields[f].levels; k++)
        k_pack3<<<grid_for(n), kThreads, 0, st>>>(sp, fields[f].dev[k], n, fields[f].levels, k);
    sp += 3 * (size_t)fields[f].levels * N;
  }
  h->snap_contacts = contacts;
  h->snap_stepped = h->stepped;
  if (contacts) {
    const int lw = 1 - h->cur;   // the buffers the last step wrote
    Dev d = make_dev(h);
    const int use_rows = h->stepped ? 1 : 0;
    k_snap_contacts<<<h->num_sms * 4, kThreads, 0, st>>>(d, h->c_pgid[lw], h->c_hist[lw], h->wh_cnt[lw],
                                                         h->wh_wall[lw], h->wh_hist[lw], h->sn_dev,
                                                         use_rows ? h->n_host + h->gcap + h->nfix : -1);
    h->sn_up = h->h_up;
  }
  CK(cudaGetLastError());
  CK(cudaEventRecord(h->ev_snap, st));
  // download on the I/O stream
  CK(cudaStreamWaitEvent(io, h->ev_snap, 0));
  CK(cudaMemcpyAsync(h->sn_n_host, s_n, sizeof(int), cudaMemcpyDeviceToHost, io));
  if (n > 0) {
    if (id) CK(cudaMemcpyAsync(id, s_id, sizeof(int) * n, cudaMemcpyDeviceToHost, io));
    if (ptype) CK(cudaMemcpyAsync(ptype, s_pt, sizeof(int) * n, cudaMemcpyDeviceToHost, io));
    if (usrmark) CK(cudaMemcpyAsync(usrmark, s_um, sizeof(int) * n, cudaMemcpyDeviceToHost, io));
    if (posR) CK(cudaMemcpyAsync(posR, s_pos, sizeof(dbl4) * n, cudaMemcpyDeviceToHost, io));
    for (int f = 0; f < 7; f++)
      if (fields[f].host)
        CK(cudaMemcpyAsync(fields[f].host, where[f], sizeof(double) * 3 * fields[f].levels * (size_t)n,
                           cudaMemcpyDeviceToHost, io));
  }
  if (contacts) k_snap_copy<<<h->num_sms * 2, kThreads, 0, io>>>(h->sn_dev, h->sn_host_dptr);
  CK(cudaGetLastError());
  CK(cudaEventRecord(h->ev_snap_done, io));
  h->snap_busy = true;
  h->snap_done = false;
  return 0;
}

int snapshot_end(sdem_h* h, int* n_out) {
  if (!h->snap_busy) return set_err(h, SDEM_E_ARG, "sdem_snapshot_end: no snapshot in flight");
  CK(cudaEventSynchronize(h->ev_snap_done));
  h->snap_busy = false;
  h->snap_done = true;
  if (n_out) *n_out = *h->sn_n_host;
  return 0;
}

// Contact records of the finished snapshot, in the restart writer's listing:
// a local pair under both particles (bucket + Head_Cp), a pair with a periodic
// image under its local particle, then each particle's wall records.
int snapshot_records(sdem_h* h, std::vector<CRec>& out) {
  if (!h->snap_done || !h->snap_contacts) return set_err(h, SDEM_E_ARG, "no finished snapshot with contacts");
  out.clear();
  const SnapContacts& v = h->sn_host;
  const int n = v.scal[0];
  const sdem_cfg& c = h->cfg;
  std::vector<int> idx_of((size_t)c.max_gid + 1, -1);
  for (int i = 0; i < n; i++) idx_of[v.gid[i]] = i;
  if (h->snap_stepped) {
    const int C = v.scal[1];
    for (int i = 0; i < C; i++) {
      const bool img = (v.og[i] & kImgFlag) != 0;
      const int o = v.og[i] & ~kImgFlag;
      const int a = idx_of[o], b = img ? -1 : idx_of[v.pg[i]];
      CRec r;
      r.t[0] = v.hs[i].x; r.t[1] = v.hs[i].y; r.t[2] = v.hs[i].z; r.vr = v.hs[i].w;
      if (a >= 0) { r.owner = a; r.partner = v.pg[i]; out.push_back(r); }
      if (b >= 0) { r.owner = b; r.partner = o; out.push_back(r); }
    }
  } else {
    // not stepped since upload: the uploaded history
    for (const auto& u : h->sn_up) {
      const int a = idx_of[u.owner], b = u.both ? idx_of[u.partner] : -1;
      CRec r;
      r.t[0] = u.hist.x; r.t[1] = u.hist.y; r.t[2] = u.hist.z; r.vr = u.hist.w;
      if (a >= 0) { r.owner = a; r.partner = u.partner; out.push_back(r); }
      if (b >= 0) { r.owner = b; r.partner = u.owner; out.push_back(r); }
    }
  }
  for (int i = 0; i < n; i++) {
    for (int j = 0; j < v.wcnt[i] && j < kKw; j++) {
      const int wi = v.wwall[(size_t)i * kKw + j];
      if (wi < 0 || wi >= h->nw) continue;
      CRec r;
      r.owner = i;
      r.partner = h->h_wall_id[wi];
      const dbl4 w = v.whist[(size_t)i * kKw + j];
      r.t[0] = w.x; r.t[1] = w.y; r.t[2] = w.z; r.vr = w.w;
      out.push_back(r);
    }
  }
  std::sort(out.begin(), out.end(), [](const CRec& a, const CRec& b) {
    return a.owner < b.owner || (a.owner == b.owner && a.partner < b.partner);
  });
  return 0;
}

int gather_contacts(sdem_h* h, std::vector<CRec>& out) {
  int rc = sync_and_check(h);
  if (rc) return rc;
  rc = snapshot_begin(h, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr,
                      nullptr, true);
  if (rc) return rc;
  rc = snapshot_end(h, nullptr);
  if (rc) return rc;
  return snapshot_records(h, out);
}

int emit_records(sdem_h* h, const std::vector<CRec>& recs, int cap, int* nc, int* owner_idx, int* partner_id,
                 double* tandelta, double* velrel) {
  (void)h;
  *nc = (int)recs.size();
  if ((int)recs.size() > cap || !owner_idx || !partner_id || !tandelta || !velrel) return 0;
  for (size_t i = 0; i < recs.size(); i++) {
    owner_idx[i] = recs[i].owner;
    partner_id[i] = recs[i].partner;
    tandelta[3 * i] = recs[i].t[0];
    tandelta[3 * i + 1] = recs[i].t[1];
    tandelta[3 * i + 2] = recs[i].t[2];
    velrel[i] = recs[i].vr;
  }
  return 0;
}
}  // namespace

int sdem_download_contacts(sdem_h* h, int cap, int* nc, int* owner_idx, int* partner_id, double* tandelta,
                           double* velrel) {
  if (!h || !nc) return SDEM_E_ARG;
  std::vector<CRec> recs;
  int rc = gather_contacts(h, recs);
  if (rc) return rc;
  return emit_records(h, recs, cap, nc, owner_idx, partner_id, tandelta, velrel);
}

int sdem_snapshot_begin(sdem_h* h, int* id, int* ptype, int* usrmark, double* posR, double* linVel, double* linAcc,
                        double* theta, double* rotVel, double* rotAcc, double* F, double* T, int want_contacts) {
  if (!h) return SDEM_E_ARG;
  if (!h->have_types) return set_err(h, SDEM_E_ARG, "sdem_snapshot_begin: call sdem_set_types first");
  return snapshot_begin(h, id, ptype, usrmark, posR, linVel, linAcc, theta, rotVel, rotAcc, F, T, want_contacts != 0);
}

int sdem_snapshot_end(sdem_h* h, int* n_out) {
  if (!h) return SDEM_E_ARG;
  // waits for the download only: steps enqueued after the snapshot keep running
  return snapshot_end(h, n_out);
}

int sdem_snapshot_contacts(sdem_h* h, int cap, int* nc, int* owner_idx, int* partner_id, double* tandelta,
                           double* velrel) {
  if (!h || !nc) return SDEM_E_ARG;
  std::vector<CRec> recs;
  int rc = snapshot_records(h, recs);
  if (rc) return rc;
  return emit_records(h, recs, cap, nc, owner_idx, partner_id, tandelta, velrel);
}

int sdem_check_restart_limit(sdem_h* h) {
  if (!h) return SDEM_E_ARG;
  std::vector<CRec> recs;
  int rc = gather_contacts(h, recs);
  if (rc) return rc;
  size_t i = 0;
  while (i < recs.size()) {
    size_t j = i;
    while (j < recs.size() && recs[j].owner == recs[i].owner) j++;
    if (j - i > 20) return set_err(h, SDEM_E_NCV20, "CL_Count_Cntctlink: so big ncv (more than 20 contacts on particle " +
                                                        std::to_string(recs[i].owner) + ")");
    i = j;
  }
  return 0;
}

int sdem_counters(sdem_h* h, int* out) {
  if (!h || !out) return SDEM_E_ARG;
  int rc = sync_and_check(h);
  if (rc) return rc;
  std::memcpy(out, h->h_counters, sizeof(int) * SDEM_CNT_SIZE);
  return 0;
}

int sdem_counters_lagged(sdem_h* h, int* out) {
  if (!h || !out) return SDEM_E_ARG;
  const long long it = h->iter_host - 1;   // the step before the last one enqueued
  const int b = (int)(it & 1);
  if (it < 1 || !h->mirror_ok || h->ev_iter[b] != it) return sdem_counters(h, out);
  CK(cudaEventSynchronize(h->ev_step[b]));
  int s[S_SIZE];
  const int* m = h->h_mirror + b * S_SIZE;
  if (m[S_ITER] != (int)it) return sdem_counters(h, out);
  std::memcpy(s, m, sizeof s);
  int rc = check_scalars(h, s);
  if (rc) return rc;
  std::memcpy(out, h->h_counters, sizeof(int) * SDEM_CNT_SIZE);
  return 0;
}

int sdem_counter_sums(sdem_h* h, long long* out) {
  if (!h || !out) return SDEM_E_ARG;
  int rc = sync_and_check(h);
  if (rc) return rc;
  unsigned long long v[3];
  CK(cudaMemcpy(v, h->ull + 2, sizeof v, cudaMemcpyDeviceToHost));
  for (int i = 0; i < 3; i++) out[i] = (long long)v[i];
  return 0;
}

int sdem_launch_count(sdem_h* h, long long* n) {
  if (!h || !n) return SDEM_E_ARG;
  *n = h->launches;
  return 0;
}

int sdem_profile_begin(sdem_h* h, int max_steps) {
  if (!h || max_steps < 1) return SDEM_E_ARG;
  for (cudaEvent_t e : h->prof_ev) cudaEventDestroy(e);
  h->prof_ev.assign((size_t)max_steps * (kPhases + 1), nullptr);
  for (auto& e : h->prof_ev) CK(cudaEventCreate(&e));
  h->prof_cap = max_steps;
  h->prof_steps = 0;
  h->prof = true;
  return 0;
}

int sdem_profile_end(sdem_h* h, int cap, double* ms, int* nsteps) {
  if (!h || !ms || !nsteps) return SDEM_E_ARG;
  CK(cudaStreamSynchronize(h->stream));
  for (int p = 0; p < cap && p < kPhases; p++) ms[p] = 0.0;
  for (int s = 0; s < h->prof_steps; s++) {
    cudaEvent_t* ev = &h->prof_ev[(size_t)s * (kPhases + 1)];
    for (int p = 0; p < kPhases && p < cap; p++) {
      float t = 0.f;
      CK(cudaEventElapsedTime(&t, ev[p], ev[p + 1]));
      ms[p] += t;
    }
  }
  *nsteps = h->prof_steps;
  for (cudaEvent_t e : h->prof_ev) cudaEventDestroy(e);
  h->prof_ev.clear();
  h->prof = false;
  h->prof_steps = h->prof_cap = 0;
  return kPhases;
}

const char* sdem_profile_phase_name(int i) { return (i >= 0 && i < kPhases) ? kPhaseNames[i] : ""; }

const char* sdem_last_error(sdem_h* h) { return h ? h->err.c_str() : g_noalloc_msg; }

/* ---- allocation-free contact count ----------------------------------------
 * Setup: the device address of the file-scope scratch array is looked up with
 * cudaGetSymbolAddress once per device, by the first call on that device with
 * it current; that first call should therefore come before any stream
 * capture.  The array is shared by every call and keeps the last call's
 * contents; the parts that must start at zero are cleared at the start of
 * each call.  Calls that overlap on the GPU (different streams or host
 * threads) race on the array. */
namespace {
NoAllocScratch* g_noalloc_addr[64] = {};

int noalloc_fail(int code, const char* msg) {
  std::snprintf(g_noalloc_msg, sizeof g_noalloc_msg, "%s", msg);
  return code;
}
}  // namespace

int sdem_count_contacts_noalloc(const sdem_cfg* cfg, double max_radius, int n, const double* d_posR,
                                unsigned long long* d_counts, void* stream) {
  g_noalloc_msg[0] = 0;
  if (!cfg || !d_counts || n < 0 || (n > 0 && !d_posR) || !(max_radius > 0.0))
    return noalloc_fail(SDEM_E_ARG, "sdem_count_contacts_noalloc: bad arguments");
  if (n > kNaMaxN)
    return noalloc_fail(SDEM_E_CAPACITY, "sdem_count_contacts_noalloc: more than SDEM_NOALLOC_MAX_PARTICLES "
                                         "(65536) particles");
  if (((uintptr_t)d_posR & 31u) != 0)
    return noalloc_fail(SDEM_E_ARG, "sdem_count_contacts_noalloc: d_posR must be 32-byte aligned");
  if (((uintptr_t)d_counts & 7u) != 0)
    return noalloc_fail(SDEM_E_ARG, "sdem_count_contacts_noalloc: d_counts must be 8-byte aligned");
  // The one-level, non-periodic search without fixed spheres is all this
  // entry point restates; the handle path covers the rest.
  if (cfg->periodic[0] || cfg->periodic[1] || cfg->periodic[2])
    return noalloc_fail(SDEM_E_UNSUPPORTED, "sdem_count_contacts_noalloc: periodic directions are not supported");
  if (cfg->cs_method != SDEM_CSM_NBS_MUNJIZA)
    return noalloc_fail(SDEM_E_UNSUPPORTED,
                        "sdem_count_contacts_noalloc: only the one-level search (CS_Method 1) is supported");
  if (cfg->n_fixed_capacity > 0)
    return noalloc_fail(SDEM_E_UNSUPPORTED, "sdem_count_contacts_noalloc: fixed spheres are not supported");
  if (!(cfg->cs_ratio >= 1.0))
    return noalloc_fail(SDEM_E_ARG, "sdem_count_contacts_noalloc: Prtcl_cs_ratio must be >= 1");
  // Init_NBSM grid (Prtcl_NBS_Munjiza.f90:66-77), as sdem_set_types builds it.
  // The extents are checked in double before any conversion to int: a tiny
  // cell or a huge or non-finite domain is refused, not cast.
  const double cell = cfg->cs_ratio * (2.0 * max_radius);
  if (!std::isfinite(cell) || !(cell > 0.0))
    return noalloc_fail(SDEM_E_ARG, "sdem_count_contacts_noalloc: the search cell is not a positive finite length");
  const double x0 = cfg->dom_min[0] - cell * 1.05, y0 = cfg->dom_min[1] - cell * 1.05, z0 = cfg->dom_min[2] - cell * 1.05;
  const double ext[3] = {std::floor((cfg->dom_max[0] + cell * 1.05 - x0) / cell) + 1.0,
                         std::floor((cfg->dom_max[1] + cell * 1.05 - y0) / cell) + 1.0,
                         std::floor((cfg->dom_max[2] + cell * 1.05 - z0) / cell) + 1.0};
  for (int a = 0; a < 3; a++) {
    if (!std::isfinite(ext[a]) || !(ext[a] >= 1.0))
      return noalloc_fail(SDEM_E_ARG, "sdem_count_contacts_noalloc: the domain gives no valid search grid");
    if (ext[a] > (double)kNaMaxCells)
      return noalloc_fail(SDEM_E_CAPACITY, "sdem_count_contacts_noalloc: the search grid has more than "
                                           "SDEM_NOALLOC_MAX_CELLS (524288) cells");
  }
  if (ext[0] * ext[1] * ext[2] > (double)kNaMaxCells)
    return noalloc_fail(SDEM_E_CAPACITY, "sdem_count_contacts_noalloc: the search grid has more than "
                                         "SDEM_NOALLOC_MAX_CELLS (524288) cells");
  const int nx = (int)ext[0], ny = (int)ext[1], nz = (int)ext[2];
  const long long ncell = (long long)nx * ny * nz;
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64)
    return noalloc_fail(SDEM_E_CUDA, "sdem_count_contacts_noalloc: no usable CUDA device");
  if (!g_noalloc_addr[dev]) {
    void* ptr = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&ptr, g_noalloc_scratch);
    if (e != cudaSuccess || !ptr)
      return noalloc_fail(SDEM_E_CUDA, "sdem_count_contacts_noalloc: cudaGetSymbolAddress of the scratch failed");
    g_noalloc_addr[dev] = (NoAllocScratch*)ptr;
  }
  NoAllocScratch* S = g_noalloc_addr[dev];
  cudaStream_t st = (cudaStream_t)stream;
  Dev d{};
  d.ncap = kNaMaxN;
  d.n_launch = n;
  d.n = &S->n;
  d.nt = &S->n;   // no periodic images here
  d.status = S->status;
  d.cell = cell;
  d.x0 = x0;
  d.y0 = y0;
  d.z0 = z0;
  d.nx = nx;
  d.ny = ny;
  d.nz = nz;
  d.ncell = ncell;
  d.posr = (dbl4*)d_posR;
  d.cell_of = S->cell_of;
  d.cell_cnt = S->cell_cnt;
  d.cell_start = S->cell_start;
  d.tmp_rank = S->tmp_rank;
  d.tmp_sorted = S->tmp_sorted;
  d.sorted = S->sorted;
  d.sortpos = S->sortpos;
  d.spos = S->spos;
  d.pf = S->pf;
  d.cdiv = fpi::divisor(cell);
  d.pf_margin = (float)(32.0 * cell * std::ldexp(1.0, -23));
  d.cellf = (float)cell;
  const int g = std::max(1, (n + kThreads - 1) / kThreads);
  k_na_begin<<<1, 1, 0, st>>>(S, n);
  if (cudaMemsetAsync(S->cell_cnt, 0, sizeof(int) * (size_t)ncell, st) != cudaSuccess)
    return noalloc_fail(SDEM_E_CUDA, "sdem_count_contacts_noalloc: cudaMemsetAsync failed");
  k_bin<<<g, kThreads, 0, st>>>(d);
  {
    const int nb = (int)std::max<long long>(1, (ncell + kScanTile - 1) / kScanTile);
    k_scan_reduce<<<nb, kScanThreads, 0, st>>>(S->cell_cnt, ncell, S->bsum);
    k_scan_blocks<<<1, 1024, 0, st>>>(S->bsum, nb);
    k_scan_apply<<<nb, kScanThreads, 0, st>>>(S->cell_cnt, ncell, S->bsum, S->cell_start, nullptr);
  }
  k_scatter<<<g, kThreads, 0, st>>>(d);
  k_cellorder<<<g, kThreads, 0, st>>>(d);
  k_na_count<<<g, kThreads, 0, st>>>(d, S->counts);
  k_na_end<<<1, 1, 0, st>>>(S, d_counts);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return noalloc_fail(SDEM_E_CUDA, cudaGetErrorString(e));
  if (cudaStreamSynchronize(st) != cudaSuccess)
    return noalloc_fail(SDEM_E_CUDA, "sdem_count_contacts_noalloc: stream synchronisation failed");
  int status = 0;
  if (cudaMemcpy(&status, &S->status[0], sizeof status, cudaMemcpyDeviceToHost) != cudaSuccess)
    return noalloc_fail(SDEM_E_CUDA, "sdem_count_contacts_noalloc: status read failed");
  if (status == SDEM_E_GRID)
    return noalloc_fail(SDEM_E_GRID, "sdem_count_contacts_noalloc: a particle is outside the padded search grid");
  if (status != 0) return noalloc_fail(status, "sdem_count_contacts_noalloc: device error");
  return 0;
}

int sdem_selftest_fp64(long long n, unsigned long long seed, long long* mismatches) {
  if (n < 0 || !mismatches) return SDEM_E_ARG;
  unsigned long long* bad = nullptr;
  if (cudaMalloc(&bad, sizeof *bad) != cudaSuccess) {
    cudaGetLastError();
    return SDEM_E_NOMEM;
  }
  unsigned long long hb = 0;
  cudaError_t e = cudaMemset(bad, 0, sizeof *bad);
  if (e == cudaSuccess) {
    k_selftest_fp64<<<1216, 256>>>(n, seed, bad);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) e = cudaMemcpy(&hb, bad, sizeof hb, cudaMemcpyDeviceToHost);
  cudaFree(bad);
  if (e != cudaSuccess) return SDEM_E_CUDA;
  *mismatches = (long long)hb;
  return 0;
}

int sdem_set_launch(sdem_h* h, int pipeline_chunks, int force_blocks_per_sm, int first_chunk_percent) {
  if (!h) return SDEM_E_ARG;
  if (pipeline_chunks < 0 || pipeline_chunks > kMaxChunks || force_blocks_per_sm < 0 || force_blocks_per_sm > 8 ||
      first_chunk_percent < -1 || first_chunk_percent > 90 || (first_chunk_percent > 0 && first_chunk_percent < 10))
    return set_err(h, SDEM_E_ARG, "sdem_set_launch: pipeline_chunks in 1..4, force_blocks_per_sm in 1..8, "
                                  "first_chunk_percent in 10..90 or -1 for the default split (0 keeps)");
  const int nc = pipeline_chunks ? pipeline_chunks : h->nchunk;
  const int fb = force_blocks_per_sm ? force_blocks_per_sm : h->force_bps;
  const int fp = first_chunk_percent == 0 ? h->first_pct : (first_chunk_percent < 0 ? 0 : first_chunk_percent);
  if (nc != h->nchunk || fb != h->force_bps || fp != h->first_pct) {
    if (h->stream) cudaStreamSynchronize(h->stream);
    drop_graph(h);   // the next step captures the new shape
    h->nchunk = nc;
    h->force_bps = fb;
    h->first_pct = fp;
  }
  return 0;
}

int sdem_get_launch(sdem_h* h, int* pipeline_chunks, int* force_blocks_per_sm, int* first_chunk_percent) {
  if (!h || !pipeline_chunks || !force_blocks_per_sm || !first_chunk_percent) return SDEM_E_ARG;
  *pipeline_chunks = h->nchunk;
  *force_blocks_per_sm = h->force_bps;
  *first_chunk_percent = h->first_pct;
  return 0;
}

int sdem_probe_fp64_peak(long long iters, double* dfma_per_s, double* ms) {
  if (iters <= 0 || !dfma_per_s || !ms) return SDEM_E_ARG;
  int dev = 0, sms = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess)
    return SDEM_E_CUDA;
  const int blocks = sms * 8, threads = 256;
  double* sink = nullptr;
  if (cudaMalloc(&sink, sizeof(double) * blocks) != cudaSuccess) {
    cudaGetLastError();
    return SDEM_E_NOMEM;
  }
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  cudaError_t e = cudaEventCreate(&e0);
  if (e == cudaSuccess) e = cudaEventCreate(&e1);
  float t = 0.f;
  if (e == cudaSuccess) {
    k_probe_dfma<<<blocks, threads>>>(iters / 8 + 1, 0.999999, 1e-7, sink);   // warm-up
    cudaEventRecord(e0);
    k_probe_dfma<<<blocks, threads>>>(iters, 0.999999, 1e-7, sink);
    cudaEventRecord(e1);
    e = cudaEventSynchronize(e1);
  }
  if (e == cudaSuccess) e = cudaGetLastError();
  if (e == cudaSuccess) e = cudaEventElapsedTime(&t, e0, e1);
  if (e0) cudaEventDestroy(e0);
  if (e1) cudaEventDestroy(e1);
  cudaFree(sink);
  if (e != cudaSuccess || !(t > 0.f)) return SDEM_E_CUDA;
  *ms = t;
  *dfma_per_s = 8.0 * (double)iters * blocks * threads / (t * 1e-3);
  return 0;
}

void sdem_destroy(sdem_h* h) {
  if (!h) return;
  if (h->stream) cudaStreamSynchronize(h->stream);
  drop_graph(h);
  for (cudaEvent_t e : h->prof_ev) cudaEventDestroy(e);
  for (void* p : h->allocs) cudaFree(p);
  if (h->h_counters) cudaFreeHost(h->h_counters);
  if (h->h_mirror) cudaFreeHost(h->h_mirror);
  if (h->h_chk) cudaFreeHost(h->h_chk);
  if (h->stage) cudaFree(h->stage);
  if (h->stream_io) cudaStreamSynchronize(h->stream_io);
  if (h->sn_state) cudaFree(h->sn_state);
  if (h->sn_ints) cudaFree(h->sn_ints);
  if (h->sn_cdev) cudaFree(h->sn_cdev);
  if (h->sn_chost) cudaFreeHost(h->sn_chost);
  if (h->sn_n_host) cudaFreeHost(h->sn_n_host);
  if (h->ev_snap) cudaEventDestroy(h->ev_snap);
  if (h->ev_snap_done) cudaEventDestroy(h->ev_snap_done);
  if (h->stream_io) cudaStreamDestroy(h->stream_io);
  if (h->stream2) cudaStreamSynchronize(h->stream2);
  if (h->ev_fork) cudaEventDestroy(h->ev_fork);
  for (int b = 0; b < 2; b++)
    if (h->ev_step[b]) cudaEventDestroy(h->ev_step[b]);
  if (h->ev_join) cudaEventDestroy(h->ev_join);
  if (h->ev_rows) cudaEventDestroy(h->ev_rows);
  for (int k = 0; k < 6; k++)
    if (h->ev_xfer[k]) cudaEventDestroy(h->ev_xfer[k]);
  for (int k = 0; k < kMaxChunks; k++)
    if (h->ev_chunk[k]) cudaEventDestroy(h->ev_chunk[k]);
  if (h->stream2) cudaStreamDestroy(h->stream2);
  if (h->stream) cudaStreamDestroy(h->stream);
  delete h;
}

// ---------------------------------------------------------------------------
// Batched form: one handle for many independent beds.  The members are split
// into groups of up to SDEM_BATCH_GROUP; a batch step is one CUDA graph per
// group, which forks from the group's stream into every member's streams,
// holds each member's step (its own kernels, grids and tables) and joins
// back, and the groups' graphs run on their own streams: small beds that fill
// few SMs each run side by side.  (512 sandboxes of 2,000-50,000 spheres: one
// graph over all of them ran at 0.59 G particle-steps/s, the members on their
// own streams at 1.66 G, groups of 8 / 16 / 32 / 64 / 128 at 1.40 / 1.67 /
// 1.72 / 1.74 / 1.51 G.)  A group graph holds two steps (each member returns to the
// buffer parity it was captured at) and is captured again when a member's
// own graphs were invalidated (an upload of another size, new walls, types or
// fixed spheres) or a member was stepped alone an odd number of times.
#ifndef SDEM_BATCH_GROUP
#define SDEM_BATCH_GROUP 64
#endif
}  // extern "C"

struct sdem_batch {
  struct Group {
    std::vector<sdem_h*> m;
    cudaStream_t stream = nullptr;
    cudaEvent_t fork = nullptr, after = nullptr;
    std::vector<cudaEvent_t> done;
    cudaGraphExec_t graph = nullptr;
    std::vector<long long> gen;        // members' graph generations at capture
    std::vector<int> cur;              // members' buffer parities at capture
    std::vector<long long> launches;   // members' kernel launches per replay
  };
  std::vector<sdem_h*> m;
  std::vector<Group> g;
  std::string err;
};

namespace {

int batch_fail(sdem_batch* b, int code, const std::string& msg) {
  b->err = msg;
  return code;
}

// Enqueues one step of every member of a group between a fork and a join on
// the group's stream (captured or not).
int batch_enqueue(sdem_batch* b, sdem_batch::Group& G) {
  if (cudaEventRecord(G.fork, G.stream) != cudaSuccess) return batch_fail(b, SDEM_E_CUDA, "batch fork event");
  for (size_t k = 0; k < G.m.size(); k++) {
    sdem_h* h = G.m[k];
    if (cudaStreamWaitEvent(h->stream, G.fork, 0) != cudaSuccess) return batch_fail(b, SDEM_E_CUDA, "batch fork");
    if (h->n_host > 0) {
      int rc = enqueue_step(h);
      if (rc) return batch_fail(b, rc, "member: " + h->err);
    }
    if (cudaEventRecord(G.done[k], h->stream) != cudaSuccess ||
        cudaStreamWaitEvent(G.stream, G.done[k], 0) != cudaSuccess)
      return batch_fail(b, SDEM_E_CUDA, "batch join");
  }
  return 0;
}

int batch_capture(sdem_batch* b, sdem_batch::Group& G) {
  if (G.graph) cudaGraphExecDestroy(G.graph);
  G.graph = nullptr;
  const size_t n = G.m.size();
  std::vector<int> cur0(n);
  std::vector<long long> l0(n);
  std::vector<bool> mok(n);
  for (size_t k = 0; k < n; k++) {
    cur0[k] = G.m[k]->cur;
    l0[k] = G.m[k]->launches;
    mok[k] = G.m[k]->mirror_ok;
  }
  cudaGraph_t g = nullptr;
  if (cudaStreamBeginCapture(G.stream, cudaStreamCaptureModeThreadLocal) != cudaSuccess)
    return batch_fail(b, SDEM_E_CUDA, "batch capture");
  int rc = batch_enqueue(b, G);
  if (!rc) rc = batch_enqueue(b, G);
  cudaError_t e = cudaStreamEndCapture(G.stream, &g);
  // capture does not execute: the members' parities and counts stay
  for (size_t k = 0; k < n; k++) {
    sdem_h* h = G.m[k];
    G.launches[k] = h->launches - l0[k];
    h->launches = l0[k];
    h->cur = cur0[k];
    h->mirror_ok = mok[k];
  }
  if (rc) {
    if (g) cudaGraphDestroy(g);
    return rc;
  }
  if (e != cudaSuccess) return batch_fail(b, SDEM_E_CUDA, std::string("batch capture: ") + cudaGetErrorString(e));
  e = cudaGraphInstantiate(&G.graph, g, 0);
  cudaGraphDestroy(g);
  if (e != cudaSuccess) {
    G.graph = nullptr;
    return batch_fail(b, SDEM_E_CUDA, std::string("batch graph: ") + cudaGetErrorString(e));
  }
  for (size_t k = 0; k < n; k++) {
    G.gen[k] = G.m[k]->graph_gen;
    G.cur[k] = cur0[k];
  }
  return 0;
}

}  // namespace

extern "C" {

int sdem_batch_create(int n, sdem_h* const* members, sdem_batch** out) {
  return sdem_batch_create_grouped(n, members, 0, out);
}

int sdem_batch_create_grouped(int n, sdem_h* const* members, int group_size, sdem_batch** out) {
  if (!out) return SDEM_E_ARG;
  *out = nullptr;
  if (n < 1 || !members || group_size < 0) return SDEM_E_ARG;
  const int gsz = group_size ? group_size : SDEM_BATCH_GROUP;
  for (int k = 0; k < n; k++)
    if (!members[k]) return SDEM_E_ARG;
  {
    std::vector<sdem_h*> sorted_m(members, members + n);
    std::sort(sorted_m.begin(), sorted_m.end());
    if (std::adjacent_find(sorted_m.begin(), sorted_m.end()) != sorted_m.end()) return SDEM_E_ARG;   // a handle joins once
  }
  sdem_batch* b = new sdem_batch();
  *out = b;
  b->m.assign(members, members + n);
  const int ng = (n + gsz - 1) / gsz;
  b->g.resize(ng);
  for (int q = 0; q < ng; q++) {
    sdem_batch::Group& G = b->g[q];
    const int lo = q * n / ng, hi = (q + 1) * n / ng;   // groups of nearly equal size
    G.m.assign(members + lo, members + hi);
    const size_t m = G.m.size();
    G.gen.assign(m, -1);
    G.cur.assign(m, -1);
    G.launches.assign(m, 0);
    G.done.assign(m, nullptr);
    if (cudaStreamCreateWithFlags(&G.stream, cudaStreamNonBlocking) != cudaSuccess ||
        cudaEventCreateWithFlags(&G.fork, cudaEventDisableTiming) != cudaSuccess ||
        cudaEventCreateWithFlags(&G.after, cudaEventDisableTiming) != cudaSuccess)
      return batch_fail(b, SDEM_E_CUDA, "batch streams/events");
    for (size_t k = 0; k < m; k++)
      if (cudaEventCreateWithFlags(&G.done[k], cudaEventDisableTiming) != cudaSuccess)
        return batch_fail(b, SDEM_E_CUDA, "batch events");
  }
  return 0;
}

int sdem_batch_step_async(sdem_batch* b, int nsteps) {
  if (!b) return SDEM_E_ARG;
  if (nsteps < 0) return batch_fail(b, SDEM_E_ARG, "sdem_batch_step: nsteps < 0");
  for (size_t k = 0; k < b->m.size(); k++) {
    sdem_h* h = b->m[k];
    if (!h->have_types) return batch_fail(b, SDEM_E_ARG, "member " + std::to_string(k) + ": call sdem_set_types first");
    if (h->prof) return batch_fail(b, SDEM_E_ARG, "member " + std::to_string(k) + ": profiling window open");
  }
  for (sdem_batch::Group& G : b->g) {
    // the group's work follows everything already enqueued on its members
    for (size_t k = 0; k < G.m.size(); k++)
      if (cudaEventRecord(G.done[k], G.m[k]->stream) != cudaSuccess ||
          cudaStreamWaitEvent(G.stream, G.done[k], 0) != cudaSuccess)
        return batch_fail(b, SDEM_E_CUDA, "batch order");
    int left = nsteps;
    while (left >= 2) {
      bool valid = G.graph != nullptr;
      for (size_t k = 0; valid && k < G.m.size(); k++)
        valid = G.gen[k] == G.m[k]->graph_gen && G.cur[k] == G.m[k]->cur;
      if (!valid) {
        int rc = batch_capture(b, G);
        if (rc) return rc;
      }
      if (cudaGraphLaunch(G.graph, G.stream) != cudaSuccess) return batch_fail(b, SDEM_E_CUDA, "batch graph launch");
      for (size_t k = 0; k < G.m.size(); k++) {
        sdem_h* h = G.m[k];
        if (h->n_host == 0) continue;
        h->launches += G.launches[k];
        h->iter_host += 2;
        h->ev_iter[0] = h->ev_iter[1] = -1;   // no per-step events inside the group graph
        h->mirror_ok = true;
        h->stepped = true;
      }
      left -= 2;
    }
    if (left == 1) {
      int rc = batch_enqueue(b, G);   // plain launches
      if (rc) return rc;
      for (sdem_h* h : G.m) {
        if (h->n_host == 0) continue;
        h->iter_host += 1;
        h->ev_iter[0] = h->ev_iter[1] = -1;
        h->stepped = true;
      }
    }
    // the members' later work (downloads, single steps) follows the group's
    if (cudaEventRecord(G.after, G.stream) != cudaSuccess) return batch_fail(b, SDEM_E_CUDA, "batch event");
    for (sdem_h* h : G.m)
      if (cudaStreamWaitEvent(h->stream, G.after, 0) != cudaSuccess) return batch_fail(b, SDEM_E_CUDA, "batch order");
  }
  return 0;
}

int sdem_batch_sync(sdem_batch* b) {
  if (!b) return SDEM_E_ARG;
  for (sdem_batch::Group& G : b->g)
    if (cudaStreamSynchronize(G.stream) != cudaSuccess) return batch_fail(b, SDEM_E_CUDA, "batch synchronisation");
  for (size_t k = 0; k < b->m.size(); k++) {
    int rc = sync_and_check(b->m[k]);
    if (rc) return batch_fail(b, rc, "member " + std::to_string(k) + ": " + b->m[k]->err);
  }
  b->err.clear();
  return 0;
}

int sdem_batch_step(sdem_batch* b, int nsteps) {
  int rc = sdem_batch_step_async(b, nsteps);
  if (rc) return rc;
  return sdem_batch_sync(b);
}

const char* sdem_batch_last_error(sdem_batch* b) { return b ? b->err.c_str() : ""; }

void sdem_batch_destroy(sdem_batch* b) {
  if (!b) return;
  for (sdem_batch::Group& G : b->g) {
    if (G.stream) cudaStreamSynchronize(G.stream);
    if (G.graph) cudaGraphExecDestroy(G.graph);
    for (cudaEvent_t e : G.done)
      if (e) cudaEventDestroy(e);
    if (G.fork) cudaEventDestroy(G.fork);
    if (G.after) cudaEventDestroy(G.after);
    if (G.stream) cudaStreamDestroy(G.stream);
  }
  delete b;
}

}  // extern "C"
