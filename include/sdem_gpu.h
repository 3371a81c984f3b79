/*
 * sdem_gpu.h -- C ABI of the GB300 (sm_103a) particle hot path of sDEM.
 *
 * One handle owns one bed on one GPU: particle state, material tables, plane
 * walls, the contact list with tangential-spring history, and the device
 * buffers/stream that advance it.  The calls replace, for one rank holding the
 * whole domain, the body of DEMS_iterate (src/DEM/Prtcl_DEMSystem.f90:214-247):
 * preIteration -> FindContacts -> FindContactsPW -> clc_Acceleration ->
 * Prtcl_Integrate -> Comm_For_Exchange (out-of-domain delete) -> RemvReleased.
 *
 * Conventions
 *   - every call returns an int status, SDEM_OK (0) on success; on failure
 *     sdem_last_error() returns a message.  Error codes mirror the abort sites
 *     of the reference (see each define).
 *   - host arrays are owned by the caller; the library copies in and out and
 *     retains no caller pointer after a call returns.
 *   - indices are 0-based; particle types and wall types are 1-based as in the
 *     reference's namelists; particle ids (GPrtcl_id) and wall ids
 *     (Base_wall_id + k) are the reference's integer ids.
 *   - vector fields use the reference's in-memory layout:
 *       posR   : 4 doubles per particle (x, y, z, radius)      -- type(real4)
 *       linVel : 3*tsize doubles per particle, Fortran (k,i) order, i.e.
 *                linVel[(i*tsize + k)*3 + c] is component c of level k
 *                of particle i                                 -- type(real3)(tsize,:)
 *       linAcc : same as linVel; rotVel/rotAcc use rsize; theta is 3 per particle.
 *   - calls are synchronous at return unless the name says _async.
 */
#ifndef SDEM_GPU_H
#define SDEM_GPU_H

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ------------------------------------------------------ */
#define SDEM_OK            0
#define SDEM_E_ARG         1  /* bad argument / call order                                   */
#define SDEM_E_CUDA        2  /* CUDA runtime error                                          */
#define SDEM_E_CL_FULL     3  /* contact container full: Prtcl_CL_and_CF.f90:166            */
#define SDEM_E_BAD_ID      4  /* id beyond the allowed range: Prtcl_CL_and_CF.f90:164       */
#define SDEM_E_NCV20       5  /* more than 20 contacts on one particle: Prtcl_CL_and_CF.f90:641 */
#define SDEM_E_GRID        6  /* particle outside the padded search grid (Prtcl_NBS_Munjiza.f90:193-198) */
#define SDEM_E_TIMEOUT     7  /* a bounded device-side wait ran out                          */
#define SDEM_E_CAPACITY    8  /* particle capacity (mlocal) exceeded                         */
#define SDEM_E_NOMEM       9  /* device allocation failed                                    */
#define SDEM_E_UNSUPPORTED 10 /* option the GPU path does not implement                      */

/* ---- enums: values are the reference's (Prtcl_Parameters.f90:13-24) ---- */
#define SDEM_CSM_NBS_MUNJIZA   1
#define SDEM_CSM_HRCHL         2   /* hierarchical NBS Munjiza (Prtcl_Hrchl_Munjiza.f90) */
#define SDEM_CFT_LSD           1
#define SDEM_CFT_NLIN          2   /* Hertz-Mindlin */
#define SDEM_CTM_CONSTANT      1
#define SDEM_CTM_VARIABLE      2
#define SDEM_PIM_FE            1
#define SDEM_PIM_AB2           2
#define SDEM_PIM_AB3           3

/* layout of one BinaryProperty record (Prtcl_Property.f90:28-41), 11 doubles */
#define SDEM_BP_RADEFF   0
#define SDEM_BP_MASSEFF  1
#define SDEM_BP_KN       2
#define SDEM_BP_KT       3
#define SDEM_BP_CN       4
#define SDEM_BP_CT       5
#define SDEM_BP_EN       6
#define SDEM_BP_ET       7
#define SDEM_BP_MUS      8
#define SDEM_BP_MUK      9
#define SDEM_BP_MUR      10
#define SDEM_BP_SIZE     11

/* layout of one PlaneWall record (Prtcl_Geometry.f90:17-33), 25 doubles + 4 ints */
#define SDEM_W_P1     0   /* 3 */
#define SDEM_W_P2     3   /* 3 */
#define SDEM_W_P3     6   /* 3 */
#define SDEM_W_P4     9   /* 3 */
#define SDEM_W_N      12  /* 3: unit normal  */
#define SDEM_W_D      15  /* 1: n.x + d = 0  */
#define SDEM_W_VEL    16  /* 3: trans_vel    */
#define SDEM_W_MIN    19  /* 3: min_point    */
#define SDEM_W_MAX    22  /* 3: max_point    */
#define SDEM_W_SIZE   25
#define SDEM_WF_BOTHSIDE  0
#define SDEM_WF_INFINITE  1
#define SDEM_WF_WALL_ID   2
#define SDEM_WF_WALL_TYPE 3
#define SDEM_WF_SIZE      4

/* counters returned by sdem_counters() */
#define SDEM_CNT_PP        0  /* numCntcts(1): exact particle-particle contacts          */
#define SDEM_CNT_PPG       1  /* numCntcts(2): particle-image pairs (periodic directions) */
#define SDEM_CNT_PPFIX     2  /* numCntcts(3): particle-fixed particle                    */
#define SDEM_CNT_PW        3  /* numCntcts(4): particle-wall                              */
#define SDEM_CNT_CNSV      4  /* num_Cnsv_cntct: conservative candidate pairs             */
#define SDEM_CNT_NLOCAL    5  /* particles in the domain after the step                   */
#define SDEM_CNT_ITER      6  /* iterNumber after the last step                           */
#define SDEM_CNT_NEXTWALL  7  /* Next_iter_update of the near-wall list                   */
#define SDEM_CNT_CNSV_CROSS 8 /* lvl_num_cnsv_cntct: cross-level candidates (CS_Method 2)  */
#define SDEM_CNT_SIZE      9

/* Configuration: the &DEMOptions fields the hot path reads
 * (Prtcl_Parameters.f90:45-95), plus the GPU's own capacities. */
typedef struct sdem_cfg {
  int    n_capacity;            /* mlocal: maximum particles                         */
  int    max_gid;               /* largest particle id that can occur (ids are 1..max_gid) */
  int    tsize, rsize;          /* AB history depth: max(PI_Method,1), max(PRI_Method,1) */
  int    cf_type;               /* SDEM_CFT_*                                        */
  int    ct_model;              /* SDEM_CTM_*                                        */
  int    pi_method, pri_method; /* SDEM_PIM_*                                        */
  int    cs_method;             /* SDEM_CSM_NBS_MUNJIZA or SDEM_CSM_HRCHL            */
  int    cntct_list_size;       /* CntctList_Size (contact records = size * mlocal)  */
  int    base_wall_id;          /* Base_wall_id                                      */
  int    wall_max_update_iter;  /* Wall_max_update_iter                              */
  int    periodic[3];           /* IsPeriodic; each periodic side > 2 search cells   */
  int    quirk_ab2_rot;         /* 1: AB2 rotation starts from linVel (Prtcl_Integration.f90:64) */
  int    max_contacts_per_particle; /* GPU row capacity per particle, 0 = default (24), <= 64; for
                                       radii ratio q = rmax/rmin, 3.63*(1+q)^2 bounds the spheres
                                       that can touch the largest one (59 at q = 3)           */
  double dt;                    /* dtDEM                                             */
  double gravity[3];
  double dom_min[3], dom_max[3];/* SimDomain_min/max (the whole domain on one rank)  */
  double cs_ratio;              /* Prtcl_cs_ratio                                    */
  double wall_neighbor_ratio;   /* Wall_neighbor_ratio                               */
  int    n_fixed_capacity;      /* numPrtclFix: most fixed spheres (0 = none)        */
  int    cs_num_levels;         /* CS_numlvls of the hierarchical search (0: from the diameter ratio) */
} sdem_cfg;

typedef struct sdem_h sdem_h;

/* Fills *cfg with the reference's defaults (Prtcl_Parameters.f90:45-95). */
void sdem_default_cfg(sdem_cfg* cfg);

/* Creates a handle on the current CUDA device; replaces the allocation steps of
 * DEMS_Initialize (Prtcl_DEMSystem.f90:58-195): GL_AllocateAllVar,
 * InitContactList (Prtcl_CL_and_CF.f90:66-103), Init_NBSM
 * (Prtcl_NBS_Munjiza.f90:57-113), InitContactSearchPW (Prtcl_ContactSearchPW.f90:49-76). */
int sdem_create(const sdem_cfg* cfg, sdem_h** out);

/* Uploads the material tables built by InitPrtclProperty/InitWallProperty
 * (Prtcl_Property.f90:62-195).  radius/mass/inertia: nT doubles (Prtcl_PureProp).
 * bnry_pp: nT*nT records of SDEM_BP_SIZE doubles, record (i,j) at ((j*nT)+i),
 * i.e. Fortran column order of Prtcl_BnryProp(i,j); bnry_pw: nT*nWT records,
 * record (i,w) at ((w*nT)+i) for PrtclWall_BnryProp(i,w). */
int sdem_set_types(sdem_h* h, int nT, const double* radius, const double* mass,
                   const double* inertia, const double* bnry_pp,
                   int nWT, const double* bnry_pw);

/* Uploads the plane walls made by G_MakeGeometry/G_add_PlaneWall
 * (Prtcl_Geometry.f90:457-637): nw records of SDEM_W_SIZE doubles and
 * SDEM_WF_SIZE ints (bothSide, isInfinite, wall_id, wall_Type). nw <= 64. */
int sdem_set_walls(sdem_h* h, int nw, const double* wall, const int* flags);

/* Uploads particles (GL arrays of Prtcl_Variables.f90:26-36).  Any of linAcc,
 * theta, rotVel, rotAcc may be NULL (zeros).  Resets the contact history and the
 * near-wall list (next step refreshes it, as after DEMS_Initialize). */
int sdem_upload_particles(sdem_h* h, int n, const int* id, const int* ptype,
                          const int* usrmark, const double* posR,
                          const double* linVel, const double* linAcc,
                          const double* theta, const double* rotVel,
                          const double* rotAcc);

/* Uploads contact history as read back from a restart file
 * (PIO_RestartCL, Prtcl_IOAndVisu.f90:296-377 -> CL_Add_RestartCntctlink,
 * Prtcl_CL_and_CF.f90:577-622): nc records (owner particle index, partner id,
 * TanDelta[3], VelRel_Init).  A particle-particle record is kept under the
 * pair (lower id, higher id); when both sides list it, the lower-id owner's
 * record is the one used, as in the reference's bucket lookup.  partner ids
 * above base_wall_id are walls. */
int sdem_upload_contacts(sdem_h* h, int nc, const int* owner_idx,
                         const int* partner_id, const double* tandelta,
                         const double* velrel);

/* Advances nsteps time steps (DEMS_iterate, Prtcl_DEMSystem.f90:201-317, without
 * its I/O).  Synchronous. */
int sdem_step(sdem_h* h, int nsteps);

/* Same, enqueued on the handle's stream without a final synchronisation.  Errors
 * raised on the device are reported by the next synchronous call. */
int sdem_step_async(sdem_h* h, int nsteps);

/* Returns the handle's cudaStream_t (as void*) so a caller can order its own
 * work or timing events with the steps. */
int sdem_get_stream(sdem_h* h, void** stream);

/* Downloads the particle state (same layouts as the upload).  *n receives the
 * particle count; any output pointer may be NULL. */
int sdem_download_particles(sdem_h* h, int* n, int* id, int* ptype, int* usrmark,
                            double* posR, double* linVel, double* linAcc,
                            double* theta, double* rotVel, double* rotAcc);

/* Downloads the contact list as the restart writer lists it
 * (CL_Gather_Cntctlink_Restart, Prtcl_CL_and_CF.f90:656-685): every
 * particle-particle contact under both particles, every wall contact under
 * its particle, each with TanDelta[3] and VelRel_Init.  Records are grouped
 * by owner index and sorted by partner id within an owner.  With cap smaller
 * than the count, nothing is written and *nc receives the count.
 * The returned ncv per particle is checked against the restart limit of 20
 * only by sdem_check_restart_limit(). */
int sdem_download_contacts(sdem_h* h, int cap, int* nc, int* owner_idx,
                           int* partner_id, double* tandelta, double* velrel);

/* SDEM_E_NCV20 when any particle has more than 20 contacts, the abort of
 * CL_Count_Cntctlink (Prtcl_CL_and_CF.f90:641,648) that the restart writer hits. */
int sdem_check_restart_limit(sdem_h* h);

/* Contact force and torque of the last step (GPrtcl_cntctForce, GPrtcl_torque),
 * 3 doubles per particle each; either may be NULL. */
int sdem_download_forces(sdem_h* h, double* F, double* T);

/* Fixed spheres (PIO_ReadFixedCoord, Prtcl_IOAndVisu.f90:164-291; FineSearch1
 * and ContactForce_PPFix, Prtcl_NBS_Munjiza.f90:478-498,
 * Prtcl_CL_and_CF.f90:200-222,803-827): nfix <= n_fixed_capacity spheres,
 * centres pos (3 doubles each), types 1..nT (radius from the type) and ids
 * above max_gid and below base_wall_id (the reference numbers them file
 * position + numPrtcl).  Spheres outside [dom_min, dom_max) are dropped, as the
 * reader does on one rank.  Call after sdem_set_types; not with periodic
 * directions (SDEM_E_UNSUPPORTED). */
int sdem_set_fixed(sdem_h* h, int nfix, const int* id, const int* ptype, const double* pos);

/* Counters of the last step, SDEM_CNT_SIZE ints (see SDEM_CNT_*). */
int sdem_counters(sdem_h* h, int* out);

/* Counters of the step before the last one enqueued, waiting for that step
 * only: a driver that enqueues step k+1 (sdem_step_async(h, 1)) and then reads
 * the counters of step k keeps the device busy while it reads them.  Device
 * errors raised up to that step are reported here.  When that step's copy is
 * not at hand (fewer than two steps since the upload, a multi-step call, a
 * call that rewrote the device scalars) this is sdem_counters. */
int sdem_counters_lagged(sdem_h* h, int* out);

/* ---- asynchronous output for the dump / restart steps ---------------------
 * Replaces the synchronous downloads before dump_visu and Write_Restart
 * (Prtcl_DEMSystem.f90:254,261; formats of Prtcl_IOAndVisu.f90:849-1031,
 * 1193-1267 unchanged).  sdem_snapshot_begin freezes, on the device, the
 * state after every step enqueued so far (a device-to-device copy of a few
 * hundred MB, well under a millisecond) and starts its download on a separate
 * copy stream; sdem_step_async calls made afterwards run while the copy
 * travels.  The host arrays take the layouts of sdem_download_particles
 * (n_capacity rows suffice) plus F and T (3 doubles per particle); any may be
 * NULL.  Page-locked host arrays let the copy run at full speed; others are
 * staged by the CUDA driver.  They must stay valid and untouched until
 * sdem_snapshot_end returns.  want_contacts != 0 also freezes the contact
 * list (history included), read after sdem_snapshot_end with
 * sdem_snapshot_contacts in the listing of sdem_download_contacts.  A new
 * sdem_snapshot_begin, sdem_download_contacts or sdem_check_restart_limit
 * first completes a snapshot still in flight and then replaces it. */
int sdem_snapshot_begin(sdem_h* h, int* id, int* ptype, int* usrmark, double* posR, double* linVel,
                        double* linAcc, double* theta, double* rotVel, double* rotAcc, double* F, double* T,
                        int want_contacts);
/* Waits for the snapshot's download; *n_out = particles in it. */
int sdem_snapshot_end(sdem_h* h, int* n_out);
/* Contact records of the last finished snapshot taken with want_contacts
 * (arguments as sdem_download_contacts). */
int sdem_snapshot_contacts(sdem_h* h, int cap, int* nc, int* owner_idx, int* partner_id, double* tandelta,
                           double* velrel);

/* ---- diagnostics (no counterpart in the reference) ---------------------- */
/* Sums since the last upload: out[0] particle-particle contacts over all
 * steps, out[1] wall contacts, out[2] steps (averages over a timed window). */
int sdem_counter_sums(sdem_h* h, long long* out);
/* Number of kernel launches this handle has issued. */
int sdem_launch_count(sdem_h* h, long long* n);
/* Starts per-phase CUDA-event timing of the next max_steps steps. */
int sdem_profile_begin(sdem_h* h, int max_steps);
/* Stops timing; ms[p] receives the summed milliseconds of phase p over the
 * timed steps (cap entries at most), *nsteps the number of timed steps.
 * Returns the number of phases (>0) or an error code (<0 never; see status). */
int sdem_profile_end(sdem_h* h, int cap, double* ms, int* nsteps);
/* Name of phase i ("" outside the range). */
const char* sdem_profile_phase_name(int i);
/* Runs the library's integer-pipe binary64 arithmetic (sqrt, division,
 * exact x*(-1/2), comparisons, floor into a grid range) against
 * the hardware instructions on n generated operand pairs on the current
 * device; *mismatches receives the number of pairs whose results differ in
 * any bit (0 expected). */
int sdem_selftest_fp64(long long n, unsigned long long seed, long long* mismatches);

/* ---- launch shape (no counterpart in the reference) -------------------------
 * The step's search/force pipeline runs in pipeline_chunks chunks of target
 * sort positions (1..4; default 2), the first of them holding
 * first_chunk_percent percent of the targets (10..90; -1: the default split,
 * where the first chunk holds as many whole waves of resident search blocks
 * as fit in an even share when that trims the share by a quarter at most,
 * else an even share, and the other chunks share the rest evenly), and
 * the force kernel with force_blocks_per_sm blocks per SM in it (1..8;
 * default 3).  Results are bit-identical for every value (every
 * order that matters is fixed by sort positions); only the speed changes,
 * which sdem_gb300/tune.py measures.  0 keeps a value; a change makes the
 * next step capture its graphs again.  sdem_get_launch reports the default
 * split as first_chunk_percent 0. */
int sdem_set_launch(sdem_h* h, int pipeline_chunks, int force_blocks_per_sm, int first_chunk_percent);
int sdem_get_launch(sdem_h* h, int* pipeline_chunks, int* force_blocks_per_sm, int* first_chunk_percent);

/* Measures the FP64 pipe: a kernel of eight independent DFMA chains per
 * thread (8 blocks of 256 threads per SM) runs `iters` iterations on the
 * current device; *dfma_per_s receives the executed DFMA per second (one DFMA
 * is two floating-point operations) and *ms the kernel's CUDA-event time. */
int sdem_probe_fp64_peak(long long iters, double* dfma_per_s, double* ms);

/* ---- allocation-free contact count (no counterpart in the reference) ------
 * For callers that cannot allocate device memory -- a host running inside
 * another framework's memory pool, or code between a pool reset and its next
 * allocation -- yet hold a particle set on the device and need its contact
 * count, e.g. to size buffers before creating a handle (sdem_create
 * allocates).  It counts, for the n particles of d_posR (device memory,
 * 4 doubles x, y, z, radius per particle, 32-byte aligned), the exact
 * particle-particle contacts (numCntcts(1)) and the candidate pairs of the
 * search (num_Cnsv_cntct) on the grid that sdem_create + sdem_set_types would
 * build from cfg and the largest radius max_radius, and writes them to
 * d_counts[0..1] (device memory).  It allocates nothing: its scratch is one
 * fixed-size device array in the library (about 7.3 MB, held by every GPU
 * that loads the library until the process exits), which limits n to
 * SDEM_NOALLOC_MAX_PARTICLES and the grid to SDEM_NOALLOC_MAX_CELLS; larger
 * inputs are refused with SDEM_E_CAPACITY.  It restates the one-level search
 * of a bed without periodic directions or fixed spheres: a cfg with
 * periodic[*] set, cs_method other than SDEM_CSM_NBS_MUNJIZA or
 * n_fixed_capacity > 0 is refused with SDEM_E_UNSUPPORTED (count such beds
 * with a handle).  A particle outside the padded grid gives SDEM_E_GRID and no
 * counts.  The first call on a device looks up the array's device address, so
 * make that first call before any stream capture.  All calls share the array
 * and it keeps the last call's contents (each call clears what must start at
 * zero): calls that overlap on the GPU (other streams or host threads) race.
 * The call is synchronous: it returns after its work on `stream` has finished
 * and its status has been read back.  On failure sdem_last_error(NULL) gives
 * the message. */
#define SDEM_NOALLOC_MAX_PARTICLES 65536
#define SDEM_NOALLOC_MAX_CELLS     524288
int sdem_count_contacts_noalloc(const sdem_cfg* cfg, double max_radius, int n, const double* d_posR,
                                unsigned long long* d_counts, void* stream);

/* Message of the last failure on this handle ("" when none); with h == NULL,
 * the last failure of sdem_count_contacts_noalloc on the calling thread. */
const char* sdem_last_error(sdem_h* h);

void sdem_destroy(sdem_h* h);

/* ---- batched form: one handle holds many independent beds ------------------
 * A batch groups handles created, configured and uploaded as usual (each with
 * its own particle count, materials, walls and domain) and advances all of
 * them together: a batch step is one CUDA graph that runs every member's step
 * on the member's own streams, so that beds too small to fill the GPU run side
 * by side.  Results equal stepping each member alone, bit for bit.  The
 * members stay usable: their downloads, counters and single steps are ordered
 * after the batch's steps.  A handle belongs to at most one batch and must
 * outlive it; sdem_batch_destroy does not destroy the members. */
typedef struct sdem_batch sdem_batch;
int sdem_batch_create(int n, sdem_h* const* members, sdem_batch** out);
/* The same with groups of at most group_size members (0: the default of 64):
 * one graph and one stream per group. */
int sdem_batch_create_grouped(int n, sdem_h* const* members, int group_size, sdem_batch** out);
/* nsteps steps of every member, without a final synchronisation */
int sdem_batch_step_async(sdem_batch* b, int nsteps);
/* waits for the batch and reports the first member error (SDEM_E_*) */
int sdem_batch_sync(sdem_batch* b);
/* sdem_batch_step_async + sdem_batch_sync */
int sdem_batch_step(sdem_batch* b, int nsteps);
const char* sdem_batch_last_error(sdem_batch* b);
void sdem_batch_destroy(sdem_batch* b);

#ifdef __cplusplus
}
#endif
#endif /* SDEM_GPU_H */
