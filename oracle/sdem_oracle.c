/*
 * sdem_oracle.c -- CPU restatement of sDEM's per-step particle hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  This file is the oracle the GB300 kernels are
 * compared with: only tests/, __graft_entry__.smoke() and bench.py's
 * CPU-baseline leg may load it.  No product code path calls it.
 *
 * It restates, single-threaded and in the reference's own order of operations,
 * the Fortran routines of GongZheng-Justin/sDEM (src/DEM/...):
 *   - NBS-Munjiza search           Prtcl_NBS_Munjiza.f90:57-113, 118-296, 302-473, 503-530
 *   - contact list + free list     Prtcl_CL_and_CF.f90:66-103, 142-168, 227-249, 256-296,
 *                                  500-572, 577-622, 656-685
 *   - force law (PP and PW)        Prtcl_ContactForce_inc.f90:1-86 via
 *                                  Prtcl_CL_and_CF.f90:732-756, 832-856
 *   - wall near list + contacts    Prtcl_ContactSearchPW.f90:49-76, 81-92, 159-235, 298-319
 *   - plane-wall geometry          Prtcl_Geometry.f90:55-109, 185-261
 *   - acceleration, integration    Prtcl_DEMSystem.f90:166-181, 322-331;
 *                                  Prtcl_Integration.f90:15-88
 *   - one rank, y pencil: periodic ghost images (PC_Comm_For_Cntct,
 *                                  Prtcl_Comm.f90:554-877), FineSearch3 + AddContactPPG +
 *                                  ContactForce_PPG (Prtcl_NBS_Munjiza.f90:358-405, 535-557;
 *                                  Prtcl_CL_and_CF.f90:173-195, 761-798)
 *   - one-rank out-of-domain delete or periodic wrap (y pencil)
 *                                  Prtcl_Comm.f90:1569-1840 with GL_copy
 *                                  (Prtcl_Variables.f90:351-373), CL_copy
 *                                  (Prtcl_CL_and_CF.f90:449-458), CSPW_copy
 *                                  (Prtcl_ContactSearchPW.f90:240-259)
 *   - binary material properties   Prtcl_Property.f90:120-143, 176-194, 200-247
 * Same linked lists, same LIFO orders, same scatter order of forces, so the
 * summation order of every particle's force equals the reference's.
 *
 * Parity status: the reference ships no tests, golden vectors or fixtures, and
 * it cannot be compiled where this project is built or measured (no Fortran
 * compiler, no MPI).  This restatement is therefore "parity unpinned" against
 * the running reference; it is pinned only by analytic known-answer tests.
 *
 * Floating point: compile with -O2 -ffp-contract=off (no FMA contraction,
 * no fast-math), which is how gfortran evaluates these expressions on x86-64
 * with default flags.  Exponentiation x**r calls libm pow, as gfortran does.
 */
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include "../include/sdem_gpu.h"


typedef struct { double x, y, z; } r3;
typedef struct { double x, y, z, w; } r4;

static const r3 zero_r3 = {0.0, 0.0, 0.0};

/* ---- Prtcl_TypeDef.f90 operators (:105-288) ---------------------------- */
static r3 r3add(r3 a, r3 b) { r3 c = {a.x + b.x, a.y + b.y, a.z + b.z}; return c; }
static r3 r3sub(r3 a, r3 b) { r3 c = {a.x - b.x, a.y - b.y, a.z - b.z}; return c; }
static r3 r3scale(r3 p, double v) { r3 c = {p.x * v, p.y * v, p.z * v}; return c; }   /* real3_prod2(_2) */
static r3 r3div(r3 p, double v) { r3 c = {p.x / v, p.y / v, p.z / v}; return c; }     /* real3_division2 */
static double r3dot(r3 a, r3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
static r3 r3cross(r3 u, r3 v) {
  r3 p = {u.y * v.z - u.z * v.y, u.z * v.x - u.x * v.z, u.x * v.y - u.y * v.x};
  return p;
}
static double r3norm(r3 p) { return sqrt(p.x * p.x + p.y * p.y + p.z * p.z); }
static r3 r4xyz(r4 a) { r3 c = {a.x, a.y, a.z}; return c; }
/* real4_nv(p1,p2): (p1-p2)/|p1-p2| with the 1e-10 guard (:268-281) */
static r3 nv_of(r3 s) {
  double normv = r3norm(s);
  if (normv > 1.0000E-10) return r3div(s, normv);
  return zero_r3;
}

/* ---- handle ------------------------------------------------------------ */
typedef struct {
  r3 p1, p2, p3, p4, trans_vel, n, min_point, max_point;
  double d;
  int bothSide, isInfinite, wall_id, wall_Type;
} wall_t;

/* one level of the hierarchical search (type lvl_Munjiza,
 * Prtcl_Hrchl_Munjiza.f90:24-47); list heads keep the reference's bounds */
struct hlvl {
  int lvl, lvl_multiple, nx, ny, nz;
  double cell_len;
  int *HeadY, *HeadX0, *HeadX, *HeadX2;   /* (0:ny+1), (0:nx+1) */
  int curr_xList_ind, curr_xList2_ind;
  int *HeadZ0, *HeadZ, *HeadZ2;           /* (0:2, 0:nz+1) as [m*(nz+2) + iz] */
  int curr_zList0_ind[3], curr_zList_ind[3], curr_zList2_ind[3];
};

typedef struct orc {
  sdem_cfg cfg;
  int err;
  char errmsg[256];
  /* tables */
  int nT, nWT;
  double *Radius, *Mass, *Inertia, *bpp, *bpw;
  int nw;
  wall_t* walls;
  /* particles, 1-based */
  int nlocal, mlocal, tsize, rsize;
  int *id, *pType, *usrMark;
  r4* PosR;
  r3 *linVel, *linAcc, *rotVel, *rotAcc; /* [(i)*size + (k-1)] with i 1-based */
  r3 *theta, *F, *T;
  /* contact list (Prtcl_CL_and_CF.f90:18-33), 1-based */
  int max_numCntcts, mBucket, NextInsert;
  int *Bucket, *id_j, *Next, *CntctStatus, *id_i, *Head_Cp, *Next_Cp;
  r3* TanDelta;
  double* VelRel_Init;
  int numCntcts[4];
  /* NBS (Prtcl_NBS_Munjiza.f90:15-35) */
  double cell_len, xst_cs, yst_cs, zst_cs;
  int nx, ny, nz, mbox;
  int *bx, *by, *bz, *NextX, *NextY, *NextZ, *HeadY, *HeadX, *HeadX0;
  /* hierarchical NBS (CS_Method=2, Prtcl_Hrchl_Munjiza.f90): levels 1-based */
  int num_lvls;
  struct hlvl* lvls;
  int* type_level;          /* CS_Hrchl_level of each type (0-based type index) */
  long long lvl_num_cnsv;   /* lvl_num_cnsv_cntct: cross-level candidates */
  /* fixed particles (GPFix_*, PIO_ReadFixedCoord, Prtcl_IOAndVisu.f90:164-291),
   * 1-based; in the search they take indices 1..nFixed, before the locals */
  int nFixed;
  int *FixId, *FixType;
  r4* FixPosR;
  /* periodic ghosts (GhostP_*, Prtcl_Variables.f90:69-73), 1-based */
  int nGhost, mGhost;
  int *GhostP_id, *GhostP_pType;
  r4* GhostP_PosR;
  r3 *GhostP_linVel, *GhostP_rotVel;
  int *HeadZ;  /* (0:1, 0:nz+1) stored [m*(nz+2) + iz] */
  int *HeadZ0; /* (0:2, 0:nz+1) */
  long long num_Cnsv;
  /* PW near list (Prtcl_ContactSearchPW.f90:19-31), 1-based */
  int *Bucket_PWCS, *id_Wall, *Next_PWCS;
  int mHead, max_near, NextInsertPW, Next_iter_update;
  double MaxWallVel, DeltaXmax1, DeltaXmax2;
  int iterNumber;
  int have_types;
} orc;

#define LV(h, k, i) ((h)->linVel[(size_t)(i) * (h)->tsize + (k)-1])
#define LA(h, k, i) ((h)->linAcc[(size_t)(i) * (h)->tsize + (k)-1])
#define RV(h, k, i) ((h)->rotVel[(size_t)(i) * (h)->rsize + (k)-1])
#define RA(h, k, i) ((h)->rotAcc[(size_t)(i) * (h)->rsize + (k)-1])

static int fail(orc* h, int code, const char* msg) {
  if (!h->err) {
    h->err = code;
    snprintf(h->errmsg, sizeof h->errmsg, "%s", msg);
  }
  return code;
}

const char* orc_last_error(orc* h) { return h->errmsg; }

static void* xcalloc(size_t n, size_t s) {
  void* p = calloc(n ? n : 1, s);
  if (!p) { fprintf(stderr, "oracle: out of memory\n"); abort(); }
  return p;
}

/* ---- Prtcl_Property.f90:200-247, clc_BnryPrtcl_Prop --------------------- */
void orc_binary_prop(int cf_type, double Ri, double Mi, double Ei, double pri,
                     double Rj, double Mj, double Ej, double prj, double mus,
                     double muk, double mur, double en, double et, int iswall,
                     double* out /* SDEM_BP_SIZE */) {
  double kappa, ShearModi, ShearModj, YoungsModEff, ShearModEff, Eta, K_hertz;
  double RadEff, MassEff;
  if (!iswall) {
    RadEff = (Ri * Rj) / (Ri + Rj);
    MassEff = (Mi * Mj) / (Mi + Mj);
  } else {
    RadEff = Ri;
    MassEff = Mi;
  }
  out[SDEM_BP_RADEFF] = RadEff;
  out[SDEM_BP_MASSEFF] = MassEff;
  out[SDEM_BP_EN] = en;
  out[SDEM_BP_ET] = et;
  out[SDEM_BP_MUS] = mus;
  out[SDEM_BP_MUK] = muk;
  out[SDEM_BP_MUR] = mur;
  ShearModi = Ei / (2.0 * (1.0 + pri));
  ShearModj = Ej / (2.0 * (1.0 + prj));
  YoungsModEff = 1.0 / ((1.0 - pri * pri) / Ei + (1.0 - prj * prj) / Ej);
  ShearModEff = 1.0 / ((2.0 - pri) / ShearModi + (2.0 - prj) / ShearModj);
  kappa = ((1.0 - pri) / ShearModi + (1.0 - prj) / ShearModj) /
          ((1.0 - 0.5 * pri) / ShearModi + (1.0 - 0.5 * prj) / ShearModj);
  kappa = fabs(kappa);
  Eta = log(en);
  Eta = Eta * Eta;
  out[SDEM_BP_KN] = out[SDEM_BP_KT] = out[SDEM_BP_CN] = out[SDEM_BP_CT] = 0.0;
  if (cf_type == SDEM_CFT_LSD) {
    const double PI = 3.141592653589793238462643383279502884;
    out[SDEM_BP_KN] = 1.2024 * pow(sqrt(MassEff) * (YoungsModEff * YoungsModEff) * RadEff, 0.4);
    out[SDEM_BP_KT] = kappa * out[SDEM_BP_KN];
    out[SDEM_BP_CN] = -2.0 * log(en) * sqrt(MassEff * out[SDEM_BP_KN]) / sqrt(PI * PI + Eta);
    out[SDEM_BP_CT] = 0.0;
  } else if (cf_type == SDEM_CFT_NLIN) {
    K_hertz = 4.0 / 3.0 * YoungsModEff * sqrt(RadEff);
    out[SDEM_BP_KN] = K_hertz;
    out[SDEM_BP_KT] = 16.0 / 3.0 * ShearModEff * sqrt(RadEff);
    out[SDEM_BP_CN] = -2.2664 * log(en) * sqrt(MassEff * K_hertz) / sqrt(Eta + 10.1354);
    out[SDEM_BP_CT] = 0.0;
  }
}

/* Prtcl_Property.f90:126-128: volume, mass and moment of inertia of one type */
void orc_pure_prop(double diameter, double density, double* radius, double* mass,
                   double* inertia) {
  const double PI = 3.141592653589793238462643383279502884;
  double R = 0.5 * diameter;
  double vol = 4.0 / 3.0 * PI * (R * R * R);
  *radius = R;
  *mass = density * vol;
  *inertia = 2.0 / 5.0 * (*mass) * (R * R);
}

/* ---- create / tables / walls ------------------------------------------- */
orc* orc_create(const sdem_cfg* cfg) {
  orc* h = (orc*)xcalloc(1, sizeof(orc));
  h->cfg = *cfg;
  h->mlocal = cfg->n_capacity;
  h->tsize = cfg->tsize;
  h->rsize = cfg->rsize;
  int m = h->mlocal;
  h->id = (int*)xcalloc(m + 1, sizeof(int));
  h->pType = (int*)xcalloc(m + 1, sizeof(int));
  h->usrMark = (int*)xcalloc(m + 1, sizeof(int));
  h->PosR = (r4*)xcalloc(m + 1, sizeof(r4));
  h->linVel = (r3*)xcalloc((size_t)(m + 1) * h->tsize, sizeof(r3));
  h->linAcc = (r3*)xcalloc((size_t)(m + 1) * h->tsize, sizeof(r3));
  h->rotVel = (r3*)xcalloc((size_t)(m + 1) * h->rsize, sizeof(r3));
  h->rotAcc = (r3*)xcalloc((size_t)(m + 1) * h->rsize, sizeof(r3));
  h->theta = (r3*)xcalloc(m + 1, sizeof(r3));
  h->F = (r3*)xcalloc(m + 1, sizeof(r3));
  h->T = (r3*)xcalloc(m + 1, sizeof(r3));
  /* CL_InitContactList, Prtcl_CL_and_CF.f90:66-103 */
  int mc = cfg->cntct_list_size * m;
  h->max_numCntcts = mc;
  h->mBucket = m;
  h->Bucket = (int*)xcalloc(m + 1, sizeof(int));
  h->id_j = (int*)xcalloc(mc + 1, sizeof(int));
  h->CntctStatus = (int*)xcalloc(mc + 1, sizeof(int));
  h->Next = (int*)xcalloc(mc + 1, sizeof(int));
  h->TanDelta = (r3*)xcalloc(mc + 1, sizeof(r3));
  h->VelRel_Init = (double*)xcalloc(mc + 1, sizeof(double));
  h->id_i = (int*)xcalloc(mc + 1, sizeof(int));
  h->Head_Cp = (int*)xcalloc(m + 1, sizeof(int));
  h->Next_Cp = (int*)xcalloc(mc + 1, sizeof(int));
  for (int i = 1; i <= mc; i++) {
    h->Next[i] = -i - 1;
    h->CntctStatus[i] = -1;
    h->Next_Cp[i] = -1;
  }
  if (mc > 0) h->Next[mc] = 0;
  h->NextInsert = 1;
  for (int i = 0; i <= m; i++) h->Head_Cp[i] = -1;
  /* InitContactSearchPW list sizes, Prtcl_ContactSearchPW.f90:56-63 */
  h->max_near = (int)(1.5 * (double)m) + 1;
  h->mHead = m;
  h->Bucket_PWCS = (int*)xcalloc(m + 1, sizeof(int));
  h->id_Wall = (int*)xcalloc(h->max_near + 1, sizeof(int));
  h->Next_PWCS = (int*)xcalloc(h->max_near + 1, sizeof(int));
  h->iterNumber = 0;
  h->Next_iter_update = 0;
  return h;
}

static void init_pwcs_list(orc* h) { /* Prtcl_ContactSearchPW.f90:81-92 */
  for (int i = 1; i <= h->mHead; i++) h->Bucket_PWCS[i] = 0;
  for (int i = 1; i <= h->max_near; i++) h->Next_PWCS[i] = -i - 1;
  h->Next_PWCS[h->max_near] = 0;
  h->NextInsertPW = 1;
}

static void realloc_pwcs_list(orc* h) { /* Prtcl_ContactSearchPW.f90:122-154 */
  int sizep = h->max_near;
  int sizen = (int)(1.2 * (double)sizep);
  h->id_Wall = (int*)realloc(h->id_Wall, (size_t)(sizen + 1) * sizeof(int));
  h->Next_PWCS = (int*)realloc(h->Next_PWCS, (size_t)(sizen + 1) * sizeof(int));
  if (!h->id_Wall || !h->Next_PWCS) abort();
  for (int i = sizep + 1; i <= sizen; i++) h->Next_PWCS[i] = -i - 1;
  h->Next_PWCS[sizen] = 0;
  h->NextInsertPW = sizep + 1;
  h->max_near = sizen;
}

/* Init_NBSM grid, Prtcl_NBS_Munjiza.f90:57-113 (one rank: subdomain = domain). */
static void init_nbsm(orc* h) {
  double maxR = 0.0;
  for (int t = 0; t < h->nT; t++) maxR = (t == 0 || h->Radius[t] > maxR) ? h->Radius[t] : maxR;
  double maxDiam = 2.0 * maxR;
  h->cell_len = h->cfg.cs_ratio * maxDiam;
  h->xst_cs = h->cfg.dom_min[0] - h->cell_len * 1.05;
  h->yst_cs = h->cfg.dom_min[1] - h->cell_len * 1.05;
  h->zst_cs = h->cfg.dom_min[2] - h->cell_len * 1.05;
  double xed_cs = h->cfg.dom_max[0] + h->cell_len * 1.05;
  double yed_cs = h->cfg.dom_max[1] + h->cell_len * 1.05;
  double zed_cs = h->cfg.dom_max[2] + h->cell_len * 1.05;
  h->nx = (int)((xed_cs - h->xst_cs) / h->cell_len) + 1;
  h->ny = (int)((yed_cs - h->yst_cs) / h->cell_len) + 1;
  h->nz = (int)((zed_cs - h->zst_cs) / h->cell_len) + 1;
  int mb = h->mlocal + (h->mGhost > 0 ? h->mGhost : 0);
  h->mbox = mb;
  free(h->bx); free(h->by); free(h->bz); free(h->NextX); free(h->NextY); free(h->NextZ);
  free(h->HeadY); free(h->HeadX); free(h->HeadX0); free(h->HeadZ); free(h->HeadZ0);
  h->bx = (int*)xcalloc(mb + 1, sizeof(int));
  h->by = (int*)xcalloc(mb + 1, sizeof(int));
  h->bz = (int*)xcalloc(mb + 1, sizeof(int));
  h->NextX = (int*)xcalloc(mb + 1, sizeof(int));
  h->NextY = (int*)xcalloc(mb + 1, sizeof(int));
  h->NextZ = (int*)xcalloc(mb + 1, sizeof(int));
  h->HeadY = (int*)xcalloc(h->ny + 1, sizeof(int));
  h->HeadX = (int*)xcalloc(h->nx + 1, sizeof(int));
  h->HeadX0 = (int*)xcalloc(h->nx + 1, sizeof(int));
  h->HeadZ = (int*)xcalloc((size_t)2 * (h->nz + 2), sizeof(int));
  h->HeadZ0 = (int*)xcalloc((size_t)3 * (h->nz + 2), sizeof(int));
  for (int i = 0; i <= h->ny; i++) h->HeadY[i] = -1;
  for (int i = 0; i <= h->nx; i++) h->HeadX[i] = h->HeadX0[i] = -1;
  for (int i = 0; i < 2 * (h->nz + 2); i++) h->HeadZ[i] = -1;
  for (int i = 0; i < 3 * (h->nz + 2); i++) h->HeadZ0[i] = -1;
  for (int i = 0; i <= mb; i++) h->NextX[i] = h->NextY[i] = h->NextZ[i] = -1;
}

static void init_hrchl(orc* h);

int orc_set_types(orc* h, int nT, const double* radius, const double* mass,
                  const double* inertia, const double* bnry_pp, int nWT,
                  const double* bnry_pw) {
  if (nT < 1 || nWT < 1) return fail(h, SDEM_E_ARG, "orc_set_types: nT, nWT must be >= 1");
  h->nT = nT;
  h->nWT = nWT;
  free(h->Radius); free(h->Mass); free(h->Inertia); free(h->bpp); free(h->bpw);
  h->Radius = (double*)xcalloc(nT, sizeof(double));
  h->Mass = (double*)xcalloc(nT, sizeof(double));
  h->Inertia = (double*)xcalloc(nT, sizeof(double));
  memcpy(h->Radius, radius, nT * sizeof(double));
  memcpy(h->Mass, mass, nT * sizeof(double));
  memcpy(h->Inertia, inertia, nT * sizeof(double));
  h->bpp = (double*)xcalloc((size_t)nT * nT * SDEM_BP_SIZE, sizeof(double));
  h->bpw = (double*)xcalloc((size_t)nT * nWT * SDEM_BP_SIZE, sizeof(double));
  memcpy(h->bpp, bnry_pp, (size_t)nT * nT * SDEM_BP_SIZE * sizeof(double));
  memcpy(h->bpw, bnry_pw, (size_t)nT * nWT * SDEM_BP_SIZE * sizeof(double));
  init_nbsm(h);
  if (h->cfg.cs_method == SDEM_CSM_HRCHL) init_hrchl(h);
  /* InitContactSearchPW, Prtcl_ContactSearchPW.f90:74-75 */
  double maxR = radius[0];
  for (int t = 1; t < nT; t++) if (radius[t] > maxR) maxR = radius[t];
  h->DeltaXmax1 = maxR * h->cfg.wall_neighbor_ratio;
  h->DeltaXmax2 = maxR * (h->cfg.wall_neighbor_ratio + 1.0);
  h->have_types = 1;
  return 0;
}

static void grow_nbs(orc* h);

/* PIO_ReadFixedCoord (Prtcl_IOAndVisu.f90:164-291) on one rank: the fixed
 * spheres inside [dom_min, dom_max) are kept in file order; ids as given (the
 * reader numbers them file position + numPrtcl, :249); the radius comes from
 * the type (:222). */
int orc_set_fixed(orc* h, int nfix, const int* id, const int* ptype, const double* pos) {
  if (!h->have_types) return fail(h, SDEM_E_ARG, "orc_set_fixed: call orc_set_types first");
  if (h->cfg.periodic[0] || h->cfg.periodic[1] || h->cfg.periodic[2])
    return fail(h, SDEM_E_UNSUPPORTED, "orc_set_fixed: the fixed spheres' periodic images are not restated");
  if (h->cfg.cs_method == SDEM_CSM_HRCHL)
    return fail(h, SDEM_E_UNSUPPORTED, "orc_set_fixed: the hierarchical search has no fixed-sphere branch");
  free(h->FixId); free(h->FixType); free(h->FixPosR);
  h->FixId = (int*)xcalloc((size_t)nfix + 1, sizeof(int));
  h->FixType = (int*)xcalloc((size_t)nfix + 1, sizeof(int));
  h->FixPosR = (r4*)xcalloc((size_t)nfix + 1, sizeof(r4));
  int k = 0;
  for (int i = 0; i < nfix; i++) {
    double x = pos[3 * i], y = pos[3 * i + 1], z = pos[3 * i + 2];
    if (ptype[i] < 1 || ptype[i] > h->nT) return fail(h, SDEM_E_ARG, "orc_set_fixed: type outside 1..nT");
    if (!(x >= h->cfg.dom_min[0] && x < h->cfg.dom_max[0] && y >= h->cfg.dom_min[1] && y < h->cfg.dom_max[1] &&
          z >= h->cfg.dom_min[2] && z < h->cfg.dom_max[2]))
      continue;
    k++;
    h->FixId[k] = id[i];
    h->FixType[k] = ptype[i];
    h->FixPosR[k] = (r4){x, y, z, h->Radius[ptype[i] - 1]};
  }
  h->nFixed = k;
  if (h->nFixed + h->nlocal + h->nGhost >= h->mbox) grow_nbs(h);
  return 0;
}

int orc_set_walls(orc* h, int nw, const double* w, const int* flags) {
  free(h->walls);
  h->nw = nw;
  h->walls = (wall_t*)xcalloc(nw > 0 ? nw : 1, sizeof(wall_t));
  double maxvel = 0.0;
  for (int k = 0; k < nw; k++) {
    const double* r = w + (size_t)k * SDEM_W_SIZE;
    wall_t* p = &h->walls[k];
    p->p1 = (r3){r[0], r[1], r[2]};
    p->p2 = (r3){r[3], r[4], r[5]};
    p->p3 = (r3){r[6], r[7], r[8]};
    p->p4 = (r3){r[9], r[10], r[11]};
    p->n = (r3){r[12], r[13], r[14]};
    p->d = r[15];
    p->trans_vel = (r3){r[16], r[17], r[18]};
    p->min_point = (r3){r[19], r[20], r[21]};
    p->max_point = (r3){r[22], r[23], r[24]};
    const int* f = flags + (size_t)k * SDEM_WF_SIZE;
    p->bothSide = f[0];
    p->isInfinite = f[1];
    p->wall_id = f[2];
    p->wall_Type = f[3];
    double v = r3norm(p->trans_vel);
    maxvel = (maxvel > v) ? maxvel : v; /* Fortran max(MaxWallVel, v) */
  }
  h->MaxWallVel = maxvel; /* Prtcl_ContactSearchPW.f90:65-73 */
  return 0;
}

/* G_add_PlaneWall derived fields (Prtcl_Geometry.f90:222-236): n, d, min, max. */
void orc_make_wall(const double* p1, const double* p2, const double* p3,
                   const double* p4, double* out /* SDEM_W_SIZE */) {
  r3 a = {p1[0], p1[1], p1[2]}, b = {p2[0], p2[1], p2[2]};
  r3 c = {p3[0], p3[1], p3[2]}, d = {p4[0], p4[1], p4[2]};
  r3 ln = r3cross(r3sub(b, a), r3sub(c, a));
  r3 n = r3div(ln, r3norm(ln));
  double dd = -(r3dot(n, a));
  /* min(p4,min(p3,min(p2,p1))): Fortran min of reals */
#define MN(u, v) ((u) < (v) ? (u) : (v))
#define MX(u, v) ((u) > (v) ? (u) : (v))
  r3 mn = {MN(d.x, MN(c.x, MN(b.x, a.x))), MN(d.y, MN(c.y, MN(b.y, a.y))), MN(d.z, MN(c.z, MN(b.z, a.z)))};
  r3 mx = {MX(d.x, MX(c.x, MX(b.x, a.x))), MX(d.y, MX(c.y, MX(b.y, a.y))), MX(d.z, MX(c.z, MX(b.z, a.z)))};
#undef MN
#undef MX
  double* o = out;
  memcpy(o + SDEM_W_P1, p1, 3 * sizeof(double));
  memcpy(o + SDEM_W_P2, p2, 3 * sizeof(double));
  memcpy(o + SDEM_W_P3, p3, 3 * sizeof(double));
  memcpy(o + SDEM_W_P4, p4, 3 * sizeof(double));
  o[SDEM_W_N] = n.x; o[SDEM_W_N + 1] = n.y; o[SDEM_W_N + 2] = n.z;
  o[SDEM_W_D] = dd;
  o[SDEM_W_MIN] = mn.x; o[SDEM_W_MIN + 1] = mn.y; o[SDEM_W_MIN + 2] = mn.z;
  o[SDEM_W_MAX] = mx.x; o[SDEM_W_MAX + 1] = mx.y; o[SDEM_W_MAX + 2] = mx.z;
}

/* ---- particles / contacts upload --------------------------------------- */
static void reset_contact_list(orc* h) {
  int mc = h->max_numCntcts;
  for (int i = 1; i <= mc; i++) {
    h->Next[i] = -i - 1;
    h->CntctStatus[i] = -1;
    h->Next_Cp[i] = -1;
    h->id_j[i] = 0;
    h->id_i[i] = 0;
  }
  if (mc > 0) h->Next[mc] = 0;
  h->NextInsert = 1;
  for (int i = 0; i <= h->mBucket; i++) { h->Bucket[i] = 0; h->Head_Cp[i] = -1; }
  memset(h->numCntcts, 0, sizeof h->numCntcts);
}

int orc_upload_particles(orc* h, int n, const int* id, const int* ptype,
                         const int* usrmark, const double* posR,
                         const double* linVel, const double* linAcc,
                         const double* theta, const double* rotVel,
                         const double* rotAcc) {
  if (n > h->mlocal) return fail(h, SDEM_E_CAPACITY, "orc_upload_particles: n > capacity");
  h->nlocal = n;
  int ts = h->tsize, rs = h->rsize;
  for (int i = 1; i <= n; i++) {
    int q = i - 1;
    h->id[i] = id[q];
    h->pType[i] = ptype[q];
    h->usrMark[i] = usrmark ? usrmark[q] : 0;
    h->PosR[i] = (r4){posR[4 * q], posR[4 * q + 1], posR[4 * q + 2], posR[4 * q + 3]};
    for (int k = 1; k <= ts; k++) {
      const double* v = linVel + ((size_t)q * ts + k - 1) * 3;
      LV(h, k, i) = (r3){v[0], v[1], v[2]};
      if (linAcc) {
        const double* a = linAcc + ((size_t)q * ts + k - 1) * 3;
        LA(h, k, i) = (r3){a[0], a[1], a[2]};
      } else LA(h, k, i) = zero_r3;
    }
    for (int k = 1; k <= rs; k++) {
      if (rotVel) {
        const double* v = rotVel + ((size_t)q * rs + k - 1) * 3;
        RV(h, k, i) = (r3){v[0], v[1], v[2]};
      } else RV(h, k, i) = zero_r3;
      if (rotAcc) {
        const double* a = rotAcc + ((size_t)q * rs + k - 1) * 3;
        RA(h, k, i) = (r3){a[0], a[1], a[2]};
      } else RA(h, k, i) = zero_r3;
    }
    h->theta[i] = theta ? (r3){theta[3 * q], theta[3 * q + 1], theta[3 * q + 2]} : zero_r3;
    h->F[i] = zero_r3;
    h->T[i] = zero_r3;
  }
  reset_contact_list(h);
  h->Next_iter_update = 0;
  return 0;
}

/* CL_Add_RestartCntctlink, Prtcl_CL_and_CF.f90:577-622, for one owner. */
/* The partner's index is the first i with id(i) == gid2, as the reference's
 * linear search finds it (Prtcl_CL_and_CF.f90:590-595); first_of[gid] holds
 * that index (0: none), built once per upload so that a restart of millions
 * of contacts does not search the particle list for each. */
static int add_restart_links(orc* h, int pid1, int ncv, const int* CntctVec,
                             const r3* tan, const double* vr, const int* first_of, int max_gid) {
  int gid1 = h->id[pid1];
  for (int j = 0; j < ncv; j++) {
    int pid2 = 0, gid2 = CntctVec[j];
    double dist = 0.0;
    if (gid2 >= 1 && gid2 <= max_gid) pid2 = first_of[gid2];
    if (pid2 > 0) {
      double dx = h->PosR[pid1].x - h->PosR[pid2].x;
      double dy = h->PosR[pid1].y - h->PosR[pid2].y;
      double dz = h->PosR[pid1].z - h->PosR[pid2].z;
      dist = sqrt(dx * dx + dy * dy + dz * dz) - 1.5 * (h->PosR[pid1].w + h->PosR[pid2].w);
      if (gid1 > gid2 && dist <= 0.0) continue;
    }
    int NextI = h->NextInsert;
    h->NextInsert = -h->Next[NextI];
    if (h->NextInsert == 0)
      return fail(h, SDEM_E_CL_FULL, "CL_Add_RestartCntctlink: The container is full and there is no space for new item");
    h->id_j[NextI] = gid2;
    h->Next[NextI] = h->Bucket[pid1];
    h->Bucket[pid1] = NextI;
    h->CntctStatus[NextI] = 2;
    h->TanDelta[NextI] = tan[j];
    h->VelRel_Init[NextI] = vr[j];
    if (pid2 > 0 && gid1 < gid2 && dist <= 0.0) {
      h->id_i[NextI] = gid1;
      h->Next_Cp[NextI] = h->Head_Cp[pid2];
      h->Head_Cp[pid2] = NextI;
    }
  }
  return 0;
}

/* Records must be grouped by owner (consecutive), as PIO_RestartCL reads them. */
int orc_upload_contacts(orc* h, int nc, const int* owner_idx, const int* partner_id,
                        const double* tandelta, const double* velrel) {
  int max_gid = 0;
  for (int i = 1; i <= h->nlocal; i++)
    if (h->id[i] > max_gid) max_gid = h->id[i];
  int* first_of = (int*)xcalloc((size_t)max_gid + 1, sizeof(int));
  for (int i = h->nlocal; i >= 1; i--)
    if (h->id[i] >= 1) first_of[h->id[i]] = i;
  int a = 0;
  while (a < nc) {
    int b = a;
    while (b < nc && owner_idx[b] == owner_idx[a]) b++;
    int ncv = b - a;
    int* vec = (int*)xcalloc(ncv, sizeof(int));
    r3* tan = (r3*)xcalloc(ncv, sizeof(r3));
    double* vr = (double*)xcalloc(ncv, sizeof(double));
    for (int j = 0; j < ncv; j++) {
      vec[j] = partner_id[a + j];
      tan[j] = (r3){tandelta[3 * (a + j)], tandelta[3 * (a + j) + 1], tandelta[3 * (a + j) + 2]};
      vr[j] = velrel[a + j];
    }
    int pid1 = owner_idx[a] + 1;
    int rc = (pid1 >= 1 && pid1 <= h->nlocal) ? add_restart_links(h, pid1, ncv, vec, tan, vr, first_of, max_gid)
                                              : fail(h, SDEM_E_ARG, "orc_upload_contacts: bad owner index");
    free(vec); free(tan); free(vr);
    if (rc) { free(first_of); return rc; }
    a = b;
  }
  free(first_of);
  return 0;
}

/* ---- contact list operations ------------------------------------------- */
/* Find_insert, Prtcl_CL_and_CF.f90:256-296 */
static void find_insert(orc* h, int bkt_id, int value, int* item1, int* item2) {
  if (bkt_id > h->mlocal) { *item1 = -1; *item2 = -1; return; }
  int n = h->Bucket[bkt_id];
  while (n > 0) {
    if (h->id_j[n] == value) { *item1 = 1; *item2 = n; return; }
    n = h->Next[n];
  }
  if (h->NextInsert == 0) { *item1 = -2; *item2 = -2; return; }
  int NextI = h->NextInsert;
  h->NextInsert = -h->Next[NextI];
  h->id_j[NextI] = value;
  h->Next[NextI] = h->Bucket[bkt_id];
  h->Bucket[bkt_id] = NextI;
  h->TanDelta[NextI] = zero_r3;
  h->VelRel_Init[NextI] = -2.0;
  *item1 = 2;
  *item2 = NextI;
}

static const double* bp_pp(orc* h, int ti, int tj) { /* Prtcl_BnryProp(ti,tj), 1-based */
  return h->bpp + ((size_t)(tj - 1) * h->nT + (ti - 1)) * SDEM_BP_SIZE;
}
static const double* bp_pw(orc* h, int ti, int wt) {
  return h->bpw + ((size_t)(wt - 1) * h->nT + (ti - 1)) * SDEM_BP_SIZE;
}

/* Prtcl_ContactForce_inc.f90:1-66: the force law shared by the PP and PW
 * wrappers.  Returns Fnij+Ftij, Moment and Mrij; updates TanDelta(ind),
 * VelRel_Init(ind). */
static void contact_force(orc* h, const double* P, r3 Veli, r3 Velj, r3 Rvei,
                          r3 Rvej, double ri, double rj, r3 Norm_v, double ovrlp,
                          int ind, r3* Fsum, r3* Moment, r3* Mrij) {
  double fn, ft, vrn, ft_fric, k_n, d_n, k_t, d_t, normTan1, normTan2, w_hat_mag, Vel_in;
  r3 Vrij, Vel_w, Vij_n, Vij_t, Ovlp_t, Fnij, Ftij, W_hat;
  double dt = h->cfg.dt;

  Vel_w = r3cross(r3add(r3scale(Rvei, ri), r3scale(Rvej, rj)), Norm_v);
  Vrij = r3add(r3sub(Veli, Velj), Vel_w);
  vrn = r3dot(Vrij, Norm_v);
  if (h->VelRel_Init[ind] < -1.0) h->VelRel_Init[ind] = fabs(vrn);

  Vij_n = r3scale(Norm_v, vrn);
  Vij_t = r3sub(Vrij, Vij_n);

  Ovlp_t = h->TanDelta[ind];
  normTan1 = r3norm(Ovlp_t);
  Ovlp_t = r3sub(Ovlp_t, r3scale(Norm_v, r3dot(Ovlp_t, Norm_v)));
  normTan2 = r3norm(Ovlp_t);
  if (normTan2 > 1.0E-10) Ovlp_t = r3scale(Ovlp_t, normTan1 / normTan2);
  else Ovlp_t = zero_r3;
  Ovlp_t = r3add(r3scale(Vij_t, dt), Ovlp_t);

  if (h->cfg.cf_type == SDEM_CFT_LSD) {
    Vel_in = (h->VelRel_Init[ind] > 0.01) ? h->VelRel_Init[ind] : 0.01; /* max(VelRel_Init,0.01) */
    k_n = -(P[SDEM_BP_KN] * pow(Vel_in, 0.4));
    d_n = -(P[SDEM_BP_CN] * pow(Vel_in, 0.2));
    fn = k_n * ovrlp + d_n * vrn;
    k_t = -(P[SDEM_BP_KT] * pow(Vel_in, 0.4));
    d_t = 0.0;
    Ftij = r3add(r3scale(Ovlp_t, k_t), r3scale(Vij_t, d_t));
  } else {
    k_n = -P[SDEM_BP_KN];
    d_n = -P[SDEM_BP_CN];
    fn = k_n * pow(ovrlp, 1.5) + d_n * pow(ovrlp, 0.25) * vrn;
    k_t = -(P[SDEM_BP_KT] * sqrt(ovrlp));
    d_t = 0.0;
    Ftij = r3add(r3scale(Ovlp_t, k_t), r3scale(Vij_t, d_t));
  }
  Fnij = r3scale(Norm_v, fn);

  ft = r3norm(Ftij);
  ft_fric = P[SDEM_BP_MUS] * fabs(fn);
  if (ft > ft_fric) {
    ft_fric = P[SDEM_BP_MUK] * fabs(fn);
    Ftij = r3scale(Ftij, ft_fric / ft);
    Ovlp_t = r3div(Ftij, k_t);
  }

  W_hat = r3sub(Rvei, Rvej);
  w_hat_mag = r3norm(W_hat);
  if (w_hat_mag > 1.0E-10) W_hat = r3div(W_hat, w_hat_mag);
  else W_hat = zero_r3;
  if (h->cfg.ct_model == SDEM_CTM_CONSTANT)
    *Mrij = r3scale(W_hat, -(P[SDEM_BP_MUR] * fabs(fn) * P[SDEM_BP_RADEFF]));
  else
    *Mrij = r3scale(W_hat, -(P[SDEM_BP_MUR] * fabs(fn) * P[SDEM_BP_RADEFF] * r3norm(Vel_w)));

  h->TanDelta[ind] = Ovlp_t;
  *Moment = r3cross(Norm_v, Ftij);
  *Fsum = r3add(Fnij, Ftij);
}

/* ContactForce_PP, Prtcl_CL_and_CF.f90:732-756 + scatter :69-74 of the include */
static void contact_force_pp(orc* h, int pid, int pjd, int ind, double ovrlp) {
  const double* P = bp_pp(h, h->pType[pid], h->pType[pjd]);
  r4 Posi = h->PosR[pid], Posj = h->PosR[pjd];
  double ri = Posi.w, rj = Posj.w;
  r3 Norm_v = nv_of(r3sub(r4xyz(Posj), r4xyz(Posi)));
  r3 S, M, Mr;
  contact_force(h, P, LV(h, 1, pid), LV(h, 1, pjd), RV(h, 1, pid), RV(h, 1, pjd), ri, rj,
                Norm_v, ovrlp, ind, &S, &M, &Mr);
  h->F[pid] = r3add(h->F[pid], S);
  h->T[pid] = r3add(r3add(h->T[pid], r3scale(M, ri)), Mr);
  h->F[pjd] = r3sub(h->F[pjd], S);
  h->T[pjd] = r3sub(r3add(h->T[pjd], r3scale(M, rj)), Mr);
}

/* ContactForce_PW, Prtcl_CL_and_CF.f90:832-856 + scatter :83-85 */
static void contact_force_pw(orc* h, int pid, int mwi, int ind, double ovrlp, r3 Norm_v) {
  const wall_t* W = &h->walls[mwi - 1];
  const double* P = bp_pw(h, h->pType[pid], W->wall_Type);
  double ri = h->PosR[pid].w;
  double rj = 1.00E20 * ri;
  Norm_v = r3scale(Norm_v, -1.0);
  r3 S, M, Mr;
  contact_force(h, P, LV(h, 1, pid), W->trans_vel, RV(h, 1, pid), zero_r3, ri, rj, Norm_v,
                ovrlp, ind, &S, &M, &Mr);
  h->F[pid] = r3add(h->F[pid], S);
  h->T[pid] = r3add(r3add(h->T[pid], r3scale(M, ri)), Mr);
}

/* CL_AddContactPP, Prtcl_CL_and_CF.f90:142-168 */
static void add_contact_pp(orc* h, int id1, int id2, double ovrlp) {
  int item1, item2;
  int gid2 = h->id[id2];
  find_insert(h, id1, gid2, &item1, &item2);
  if (item1 > 0) {
    h->CntctStatus[item2] = item1;
    h->numCntcts[0]++;
    contact_force_pp(h, id1, id2, item2, ovrlp);
    h->id_i[item2] = h->id[id1];
    h->Next_Cp[item2] = h->Head_Cp[id2];
    h->Head_Cp[id2] = item2;
  } else if (item1 == -1) {
    fail(h, SDEM_E_BAD_ID, "CL_AddContactPP: The inserted item's id is greater than allowed value");
  } else {
    fail(h, SDEM_E_CL_FULL, "CL_AddContactPP: The container is full and there is no space for new item");
  }
}

/* CL_AddContactPW, Prtcl_CL_and_CF.f90:227-249 */
static void add_contact_pw(orc* h, int id1, int id2, double ovrlp, r3 nv) {
  int item1, item2;
  int wid = h->walls[id2 - 1].wall_id;
  find_insert(h, id1, wid, &item1, &item2);
  if (item1 > 0) {
    h->CntctStatus[item2] = item1;
    h->numCntcts[3]++;
    contact_force_pw(h, id1, id2, item2, ovrlp, nv);
  } else if (item1 == -1) {
    fail(h, SDEM_E_BAD_ID, "CL_AddContactPW: The inserted item's id is greater than allowed value");
  } else {
    fail(h, SDEM_E_CL_FULL, "CL_AddContactPW: The container is full and there is no space for new item");
  }
}

/* CL_PreIteration, Prtcl_CL_and_CF.f90:560-572 */
static void cl_pre_iteration(orc* h) {
  memset(h->numCntcts, 0, sizeof h->numCntcts);
  for (int i = 1; i <= h->max_numCntcts; i++)
    if (h->CntctStatus[i] > 0) h->CntctStatus[i] = -2;
  for (int i = 0; i <= h->mBucket; i++) h->Head_Cp[i] = -1;
  for (int i = 1; i <= h->max_numCntcts; i++) h->Next_Cp[i] = -1;
}

/* CL_RemvReleased, Prtcl_CL_and_CF.f90:500-555 */
static void cl_remv_released(orc* h) {
  for (int pid = 1; pid <= h->nlocal; pid++) {
    int prev = 0, n = h->Bucket[pid];
    while (n > 0) {
      int NextI = h->Next[n];
      if (h->CntctStatus[n] == -2) {
        if (prev == 0) h->Bucket[pid] = NextI;
        else h->Next[prev] = NextI;
        h->CntctStatus[n] = -1;
        h->Next[n] = -h->NextInsert;
        h->NextInsert = n;
      } else {
        prev = n;
      }
      n = NextI;
    }
    n = h->Head_Cp[pid];
    while (n > 0) {
      if (h->CntctStatus[n] == 3) {
        h->Next[n] = h->Bucket[pid];
        h->Bucket[pid] = n;
        h->id_j[n] = h->id_i[n];
        h->CntctStatus[n] = 2;
      }
      n = h->Next_Cp[n];
    }
  }
  for (int pid = 1; pid <= h->max_numCntcts; pid++) {
    if (h->CntctStatus[pid] == 3) {
      h->CntctStatus[pid] = -1;
      h->Next[pid] = -h->NextInsert;
      h->NextInsert = pid;
    }
  }
}

/* ---- NBS-Munjiza (Prtcl_NBS_Munjiza.f90) ------------------------------- */
#define HZ(h, m, iz) ((h)->HeadZ[(m) * ((h)->nz + 2) + (iz)])
#define HZ0(h, m, iz) ((h)->HeadZ0[(m) * ((h)->nz + 2) + (iz)])

/* ---- periodic ghosts: PC_Comm_For_Cntct, y pencil, one rank --------------- */
static void grow_nbs(orc* h);

static void ghost_reserve(orc* h, int ng) {
  if (ng <= h->mGhost) return;
  int m = ng + ng / 2 + 16;
  h->GhostP_id = (int*)realloc(h->GhostP_id, (size_t)(m + 1) * sizeof(int));
  h->GhostP_pType = (int*)realloc(h->GhostP_pType, (size_t)(m + 1) * sizeof(int));
  h->GhostP_PosR = (r4*)realloc(h->GhostP_PosR, (size_t)(m + 1) * sizeof(r4));
  h->GhostP_linVel = (r3*)realloc(h->GhostP_linVel, (size_t)(m + 1) * sizeof(r3));
  h->GhostP_rotVel = (r3*)realloc(h->GhostP_rotVel, (size_t)(m + 1) * sizeof(r3));
  if (!h->GhostP_id || !h->GhostP_pType || !h->GhostP_PosR || !h->GhostP_linVel || !h->GhostP_rotVel) abort();
  h->mGhost = m;
}

static void ghost_from_local(orc* h, int ng, int i) {
  h->GhostP_id[ng] = h->id[i];
  h->GhostP_pType[ng] = h->pType[i];
  h->GhostP_PosR[ng] = h->PosR[i];
  h->GhostP_linVel[ng] = LV(h, 1, i);
  h->GhostP_rotVel[ng] = RV(h, 1, i);
}

static void ghost_from_ghost(orc* h, int ng, int i) {
  h->GhostP_id[ng] = h->GhostP_id[i];
  h->GhostP_pType[ng] = h->GhostP_pType[i];
  h->GhostP_PosR[ng] = h->GhostP_PosR[i];
  h->GhostP_linVel[ng] = h->GhostP_linVel[i];
  h->GhostP_rotVel[ng] = h->GhostP_rotVel[i];
}

/* Prtcl_Comm.f90:554-877 (CASE y_axis) with every neighbour rank equal to this
 * rank in the periodic directions: the ghost images within LenForCS (one
 * search cell) of a periodic boundary, created in the reference's order --
 * y first from the locals, then +x, -x, +z, -z each from the ghosts made so
 * far and then from the locals. */
static void comm_for_cntct(orc* h) {
  const double L = h->cell_len;  /* LenForCS = Prtcl_cs_ratio * maxD */
  const double* mn = h->cfg.dom_min;
  const double* mx = h->cfg.dom_max;
  const double Lx = mx[0] - mn[0], Ly = mx[1] - mn[1], Lz = mx[2] - mn[2];
  int ng = 0, ngp;
  if (h->cfg.periodic[1]) {
    for (int i = 1; i <= h->nlocal; i++) {
      double py = h->PosR[i].y;
      if (py <= mn[1] + L) { ghost_reserve(h, ng + 1); ng++; ghost_from_local(h, ng, i); h->GhostP_PosR[ng].y = py + Ly; }
      if (py >= mx[1] - L) { ghost_reserve(h, ng + 1); ng++; ghost_from_local(h, ng, i); h->GhostP_PosR[ng].y = py - Ly; }
    }
  }
  if (h->cfg.periodic[0]) {
    ngp = ng;
    for (int i = 1; i <= ngp; i++) {
      double px = h->GhostP_PosR[i].x;
      if (px >= mx[0] - L) { ghost_reserve(h, ng + 1); ng++; ghost_from_ghost(h, ng, i); h->GhostP_PosR[ng].x = px - Lx; }
    }
    for (int i = 1; i <= h->nlocal; i++) {
      double px = h->PosR[i].x;
      if (px >= mx[0] - L) { ghost_reserve(h, ng + 1); ng++; ghost_from_local(h, ng, i); h->GhostP_PosR[ng].x = px - Lx; }
    }
    ngp = ng;
    for (int i = 1; i <= ngp; i++) {
      double px = h->GhostP_PosR[i].x;
      if (px <= mn[0] + L && px >= mn[0]) { ghost_reserve(h, ng + 1); ng++; ghost_from_ghost(h, ng, i); h->GhostP_PosR[ng].x = px + Lx; }
    }
    for (int i = 1; i <= h->nlocal; i++) {
      double px = h->PosR[i].x;
      if (px <= mn[0] + L && px >= mn[0]) { ghost_reserve(h, ng + 1); ng++; ghost_from_local(h, ng, i); h->GhostP_PosR[ng].x = px + Lx; }
    }
  }
  if (h->cfg.periodic[2]) {
    ngp = ng;
    for (int i = 1; i <= ngp; i++) {
      double pz = h->GhostP_PosR[i].z;
      if (pz >= mx[2] - L) { ghost_reserve(h, ng + 1); ng++; ghost_from_ghost(h, ng, i); h->GhostP_PosR[ng].z = pz - Lz; }
    }
    for (int i = 1; i <= h->nlocal; i++) {
      double pz = h->PosR[i].z;
      if (pz >= mx[2] - L) { ghost_reserve(h, ng + 1); ng++; ghost_from_local(h, ng, i); h->GhostP_PosR[ng].z = pz - Lz; }
    }
    ngp = ng;
    for (int i = 1; i <= ngp; i++) {
      double pz = h->GhostP_PosR[i].z;
      if (pz <= mn[2] + L && pz >= mn[2]) { ghost_reserve(h, ng + 1); ng++; ghost_from_ghost(h, ng, i); h->GhostP_PosR[ng].z = pz + Lz; }
    }
    for (int i = 1; i <= h->nlocal; i++) {
      double pz = h->PosR[i].z;
      if (pz <= mn[2] + L && pz >= mn[2]) { ghost_reserve(h, ng + 1); ng++; ghost_from_local(h, ng, i); h->GhostP_PosR[ng].z = pz + Lz; }
    }
  }
  h->nGhost = ng;
  if (h->nFixed + h->nlocal + ng >= h->mbox) grow_nbs(h);
}

/* ContactForce_PPG, Prtcl_CL_and_CF.f90:761-798: force on the local particle only */
static void contact_force_ppg(orc* h, int pid, int pjd, int ind, double ovrlp) {
  const double* P = bp_pp(h, h->pType[pid], h->GhostP_pType[pjd]);
  r3 S, M, Mr;
  if (h->id[pid] < h->GhostP_id[pjd]) {
    r4 Posi = h->PosR[pid], Posj = h->GhostP_PosR[pjd];
    double ri = Posi.w, rj = Posj.w;
    r3 Norm_v = nv_of(r3sub(r4xyz(Posj), r4xyz(Posi)));
    contact_force(h, P, LV(h, 1, pid), h->GhostP_linVel[pjd], RV(h, 1, pid), h->GhostP_rotVel[pjd], ri, rj,
                  Norm_v, ovrlp, ind, &S, &M, &Mr);
    h->F[pid] = r3add(h->F[pid], S);
    h->T[pid] = r3add(r3add(h->T[pid], r3scale(M, ri)), Mr);
  } else {
    r4 Posi = h->GhostP_PosR[pjd], Posj = h->PosR[pid];
    double ri = Posi.w, rj = Posj.w;
    r3 Norm_v = nv_of(r3sub(r4xyz(Posj), r4xyz(Posi)));
    contact_force(h, P, h->GhostP_linVel[pjd], LV(h, 1, pid), h->GhostP_rotVel[pjd], RV(h, 1, pid), ri, rj,
                  Norm_v, ovrlp, ind, &S, &M, &Mr);
    h->F[pid] = r3sub(h->F[pid], S);
    h->T[pid] = r3sub(r3add(h->T[pid], r3scale(M, rj)), Mr);
  }
}

/* CL_AddContactPPG, Prtcl_CL_and_CF.f90:173-195 */
static void add_contact_ppg(orc* h, int id1, int id2, double ovrlp) {
  int item1, item2;
  int gid2 = h->GhostP_id[id2];
  find_insert(h, id1, gid2, &item1, &item2);
  if (item1 > 0) {
    h->CntctStatus[item2] = item1;
    h->numCntcts[1]++;
    contact_force_ppg(h, id1, id2, item2, ovrlp);
  } else if (item1 == -1) {
    fail(h, SDEM_E_BAD_ID, "CL_AddContactPPG: The inserted item's id is greater than allowed value");
  } else {
    fail(h, SDEM_E_CL_FULL, "CL_AddContactPPG: The container is full and there is no space for new item");
  }
}

/* NBSM_FineSearch3, Prtcl_NBS_Munjiza.f90:535-557 (pid2 is the search index of a ghost) */
static void fine_search3(orc* h, int pid1, int pid2) {
  int gid = pid2 - h->nlocal;
  double dx, dy, dz, dr, d2sum, dr2, ovrlp;
  dr = h->PosR[pid1].w + h->GhostP_PosR[gid].w;
  dr2 = dr * dr;
  dx = h->PosR[pid1].x - h->GhostP_PosR[gid].x;
  d2sum = dx * dx;
  if (d2sum > dr2) return;
  dy = h->PosR[pid1].y - h->GhostP_PosR[gid].y;
  d2sum = dy * dy + d2sum;
  if (d2sum > dr2) return;
  dz = h->PosR[pid1].z - h->GhostP_PosR[gid].z;
  d2sum = dz * dz + d2sum;
  if (d2sum > dr2) return;
  ovrlp = dr - sqrt(d2sum);
  add_contact_ppg(h, pid1, gid, ovrlp);
}

/* NBSM_FineSearch2, :503-530 */
static void fine_search2(orc* h, int pid1, int pid2) {
  double dx, dy, dz, dr, d2sum, dr2, ovrlp;
  dr = h->PosR[pid1].w + h->PosR[pid2].w;
  dr2 = dr * dr;
  dx = h->PosR[pid1].x - h->PosR[pid2].x;
  d2sum = dx * dx;
  if (d2sum > dr2) return;
  dy = h->PosR[pid1].y - h->PosR[pid2].y;
  d2sum = dy * dy + d2sum;
  if (d2sum > dr2) return;
  dz = h->PosR[pid1].z - h->PosR[pid2].z;
  d2sum = dz * dz + d2sum;
  if (d2sum > dr2) return;
  ovrlp = dr - sqrt(d2sum);
  if (h->id[pid1] < h->id[pid2]) add_contact_pp(h, pid1, pid2, ovrlp);
  else add_contact_pp(h, pid2, pid1, ovrlp);
}

/* ContactForce_PPFix, Prtcl_CL_and_CF.f90:803-827: the moving particle is i,
 * the fixed one j (zero velocities); force and torque on i only (the
 * ContactForce_PPFix_W branch of Prtcl_ContactForce_inc.f90:83-86). */
static void contact_force_ppfix(orc* h, int pid, int f, int ind, double ovrlp) {
  const double* P = bp_pp(h, h->pType[pid], h->FixType[f]);
  r4 Posi = h->PosR[pid], Posj = h->FixPosR[f];
  double ri = Posi.w, rj = Posj.w;
  r3 Norm_v = nv_of(r3sub(r4xyz(Posj), r4xyz(Posi)));
  r3 S, M, Mr;
  contact_force(h, P, LV(h, 1, pid), zero_r3, RV(h, 1, pid), zero_r3, ri, rj, Norm_v, ovrlp, ind, &S, &M, &Mr);
  h->F[pid] = r3add(h->F[pid], S);
  h->T[pid] = r3add(r3add(h->T[pid], r3scale(M, ri)), Mr);
}

/* CL_AddContactPPFix, Prtcl_CL_and_CF.f90:200-222 */
static void add_contact_ppfix(orc* h, int id1, int f, double ovrlp) {
  int item1, item2;
  find_insert(h, id1, h->FixId[f], &item1, &item2);
  if (item1 > 0) {
    h->CntctStatus[item2] = item1;
    h->numCntcts[2]++;
    contact_force_ppfix(h, id1, f, item2, ovrlp);
  } else if (item1 == -1) {
    fail(h, SDEM_E_BAD_ID, "CL_AddContactPPFix: The inserted item's id is greater than allowed value");
  } else {
    fail(h, SDEM_E_CL_FULL, "CL_AddContactPPFix: The container is full and there is no space for new item");
  }
}

/* NBSM_FineSearch1, Prtcl_NBS_Munjiza.f90:478-498 (pid1 a local, f a fixed particle) */
static void fine_search1(orc* h, int pid1, int f) {
  double dx, dy, dz, dr, d2sum, dr2, ovrlp;
  dr = h->PosR[pid1].w + h->FixPosR[f].w;
  dr2 = dr * dr;
  dx = h->PosR[pid1].x - h->FixPosR[f].x;
  d2sum = dx * dx;
  if (d2sum > dr2) return;
  dy = h->PosR[pid1].y - h->FixPosR[f].y;
  d2sum = dy * dy + d2sum;
  if (d2sum > dr2) return;
  dz = h->PosR[pid1].z - h->FixPosR[f].z;
  d2sum = dz * dz + d2sum;
  if (d2sum > dr2) return;
  ovrlp = dr - sqrt(d2sum);
  add_contact_ppfix(h, pid1, f, ovrlp);
}

/* NBSM_clcBoxIndex, :163-212, and the fixed particles' indices of Init_NBSM
 * (:104-109).  Search index s: 1..nFixed fixed, then the locals, then the
 * ghosts (nFixedAndlocal = nFixed + nlocal, :127-129). */
static int clc_box_index(orc* h) {
  const int nf = h->nFixed, nfl = h->nFixed + h->nlocal;
  for (int i = 1; i <= nfl + h->nGhost; i++) {
    r4 P = (i <= nf) ? h->FixPosR[i] : (i <= nfl) ? h->PosR[i - nf] : h->GhostP_PosR[i - nfl];
    double rpdx = P.x - h->xst_cs;
    double rpdy = P.y - h->yst_cs;
    double rpdz = P.z - h->zst_cs;
    h->bx[i] = (int)floor(rpdx / h->cell_len) + 1;
    h->by[i] = (int)floor(rpdy / h->cell_len) + 1;
    h->bz[i] = (int)floor(rpdz / h->cell_len) + 1;
    /* The reference indexes its head arrays with these without a check; a
     * particle outside the padded grid is an error here. */
    if (h->bx[i] < 1 || h->bx[i] > h->nx || h->by[i] < 1 || h->by[i] > h->ny ||
        h->bz[i] < 1 || h->bz[i] > h->nz)
      return fail(h, SDEM_E_GRID, "NBSM_clcBoxIndex: particle outside the search grid");
  }
  return 0;
}

static void build_y_list(orc* h) { /* :217-229 */
  for (int i = 1; i <= h->ny; i++) h->HeadY[i] = -1;
  for (int i = 1; i <= h->nFixed + h->nlocal + h->nGhost; i++) {
    int iy = h->by[i];
    h->NextY[i] = h->HeadY[iy];
    h->HeadY[iy] = i;
  }
}

static void build_x_list(orc* h, int iy) { /* :234-250 */
  for (int i = 1; i <= h->nx; i++) h->HeadX[i] = -1;
  int n = h->HeadY[iy];
  while (n != -1) {
    int ix = h->bx[n];
    h->NextX[n] = h->HeadX[ix];
    h->HeadX[ix] = n;
    n = h->NextY[n];
  }
}

static void build_z_list(orc* h, int ix, int m) { /* :255-272 */
  for (int iz = 0; iz <= h->nz + 1; iz++) HZ(h, m, iz) = -1;
  int n = h->HeadX[ix + m - 1];
  while (n != -1) {
    int iz = h->bz[n];
    h->NextZ[n] = HZ(h, m, iz);
    HZ(h, m, iz) = n;
    n = h->NextX[n];
  }
}

static void build_z_list0(orc* h, int ix, int m) { /* :277-296 */
  for (int iz = 0; iz <= h->nz + 1; iz++) HZ0(h, m, iz) = -1;
  int ixm = ix + m - 1;
  if (ixm > h->nx) return;
  int n = h->HeadX0[ixm];
  while (n != -1) {
    int iz = h->bz[n];
    h->NextZ[n] = HZ0(h, m, iz);
    HZ0(h, m, iz) = n;
    n = h->NextX[n];
  }
}

/* NBSM_LoopNBSMask, :302-473.  Search indices: s <= nf fixed, s > nfl ghost,
 * else local (local pid = s - nf, ghost index for fine_search3 = s - nf).
 * A fixed or ghost target pairs with local particles only (FineSearch1/3 with
 * the local first); a local target with everything (:406-469). */
static void loop_nbs_mask(orc* h, int iz) {
  const int nf = h->nFixed, nfl = h->nFixed + h->nlocal;
  int m = HZ(h, 1, iz);
  while (m != -1) {
    if (m <= nf) {
#define FIXED_VISIT(start) do { int n_ = (start); while (n_ != -1) { if (n_ <= nfl && n_ > nf) { fine_search1(h, n_ - nf, m); h->num_Cnsv++; } n_ = h->NextZ[n_]; } } while (0)
      FIXED_VISIT(h->NextZ[m]);
      FIXED_VISIT(HZ(h, 1, iz - 1));
      for (int i = -1; i <= 1; i++) FIXED_VISIT(HZ(h, 0, iz + i));
      for (int lx = 0; lx <= 2; lx++)
        for (int i = -1; i <= 1; i++) FIXED_VISIT(HZ0(h, lx, iz + i));
#undef FIXED_VISIT
    } else if (m > nfl) {
#define GHOST_VISIT(start) do { int n_ = (start); while (n_ != -1) { if (n_ <= nfl && n_ > nf) { fine_search3(h, n_ - nf, m - nf); h->num_Cnsv++; } n_ = h->NextZ[n_]; } } while (0)
      GHOST_VISIT(h->NextZ[m]);
      GHOST_VISIT(HZ(h, 1, iz - 1));
      for (int i = -1; i <= 1; i++) GHOST_VISIT(HZ(h, 0, iz + i));
      for (int lx = 0; lx <= 2; lx++)
        for (int i = -1; i <= 1; i++) GHOST_VISIT(HZ0(h, lx, iz + i));
#undef GHOST_VISIT
    } else {
#define LOCAL_VISIT(start) do { int n_ = (start); while (n_ != -1) { if (n_ <= nf) fine_search1(h, m - nf, n_); else if (n_ > nfl) fine_search3(h, m - nf, n_ - nf); else fine_search2(h, m - nf, n_ - nf); h->num_Cnsv++; n_ = h->NextZ[n_]; } } while (0)
      LOCAL_VISIT(h->NextZ[m]);
      LOCAL_VISIT(HZ(h, 1, iz - 1));
      for (int i = -1; i <= 1; i++) LOCAL_VISIT(HZ(h, 0, iz + i));
      for (int lx = 0; lx <= 2; lx++)
        for (int i = -1; i <= 1; i++) LOCAL_VISIT(HZ0(h, lx, iz + i));
#undef LOCAL_VISIT
    }
    m = h->NextZ[m];
  }
}

/* NBSM_clcBoxIndex regrow (:172-189): room for locals + ghosts */
static void grow_nbs(orc* h) {
  int sizen = (int)(1.2 * (double)h->mbox);
  int need = h->nFixed + h->nlocal + h->nGhost + 1;
  if (sizen < need) sizen = need;
  free(h->bx); free(h->by); free(h->bz); free(h->NextX); free(h->NextY); free(h->NextZ);
  h->bx = (int*)xcalloc(sizen + 1, sizeof(int));
  h->by = (int*)xcalloc(sizen + 1, sizeof(int));
  h->bz = (int*)xcalloc(sizen + 1, sizeof(int));
  h->NextX = (int*)xcalloc(sizen + 1, sizeof(int));
  h->NextY = (int*)xcalloc(sizen + 1, sizeof(int));
  h->NextZ = (int*)xcalloc(sizen + 1, sizeof(int));
  h->mbox = sizen;
}

/* NBSM_ContactSearch, :118-158 */
static int nbsm_contact_search(orc* h) {
  h->num_Cnsv = 0;
  if (h->nlocal == 0) return 0;
  if (clc_box_index(h)) return h->err;
  build_y_list(h);
  for (int i = 1; i <= h->nx; i++) h->HeadX0[i] = -1;
  for (int iy = 1; iy <= h->ny; iy++) {
    build_x_list(h, iy);
    if (h->HeadY[iy] != -1) {
      for (int iz = 0; iz <= h->nz + 1; iz++) { HZ(h, 0, iz) = -1; HZ0(h, 0, iz) = -1; }
      build_z_list0(h, 1, 1);
      for (int ix = 1; ix <= h->nx; ix++) {
        build_z_list(h, ix, 1);
        build_z_list0(h, ix, 2);
        if (h->HeadX[ix] != -1)
          for (int iz = 1; iz <= h->nz; iz++) loop_nbs_mask(h, iz);
        for (int iz = 0; iz <= h->nz + 1; iz++) {
          HZ(h, 0, iz) = HZ(h, 1, iz);
          HZ0(h, 0, iz) = HZ0(h, 1, iz);
          HZ0(h, 1, iz) = HZ0(h, 2, iz);
        }
        if (h->err) return h->err;
      }
    }
    for (int i = 1; i <= h->nx; i++) h->HeadX0[i] = h->HeadX[i];
  }
  return h->err;
}

/* ---- hierarchical NBS (CS_Method = 2), Prtcl_Hrchl_Munjiza.f90 ------------
 * A line-by-line restatement, list quirks included: BuildXList2 records its
 * row in curr_xList_ind (:453), so curr_xList2_ind stays -1 and the
 * "already built" test of BuildXList2 never holds.  Search indices: locals
 * 1..nlocal, ghosts after them (no fixed particles in this search). */
#define HLZ(L, arr, m, iz) ((L)->arr[(m) * ((L)->nz + 2) + (iz)])

static void hlvl_free(struct hlvl* L) {
  free(L->HeadY); free(L->HeadX0); free(L->HeadX); free(L->HeadX2);
  free(L->HeadZ0); free(L->HeadZ); free(L->HeadZ2);
}

/* Init_Munjiza_Hrchl, :78-218.  Every type of the table counts as populated
 * (nPrtcl_in_Bin > 0): a level without particles has empty lists and finds
 * nothing, so dropping it or keeping it gives the same contacts. */
static void init_hrchl(orc* h) {
  for (int k = 1; k <= h->num_lvls; k++) hlvl_free(&h->lvls[k]);
  free(h->lvls); free(h->type_level);
  double maxD = 0.0, minD = 0.0;
  for (int t = 0; t < h->nT; t++) {
    double d = 2.0 * h->Radius[t];
    if (t == 0 || d > maxD) maxD = d;
    if (t == 0 || d < minD) minD = d;
  }
  int dmax_min = (int)(maxD / minD);
  int numLevels;
  if (h->cfg.cs_num_levels > 0) numLevels = h->cfg.cs_num_levels;
  else if (dmax_min <= 1) numLevels = 1;
  else if (dmax_min <= 3) numLevels = 2;
  else if (dmax_min <= 7) numLevels = 3;
  else if (dmax_min <= 15) numLevels = 4;
  else if (dmax_min <= 31) numLevels = 5;
  else numLevels = 6;
  h->type_level = (int*)xcalloc(h->nT, sizeof(int));
  h->lvls = (struct hlvl*)xcalloc((size_t)numLevels + 1, sizeof(struct hlvl));
  double cell_len = h->cfg.cs_ratio * maxD;
  double xst = h->cfg.dom_min[0] - cell_len * 1.05, yst = h->cfg.dom_min[1] - cell_len * 1.05;
  double zst = h->cfg.dom_min[2] - cell_len * 1.05;
  double xed = h->cfg.dom_max[0] + cell_len * 1.05, yed = h->cfg.dom_max[1] + cell_len * 1.05;
  double zed = h->cfg.dom_max[2] + cell_len * 1.05;
  h->xst_cs = xst; h->yst_cs = yst; h->zst_cs = zst;
  int nx = (int)((xed - xst) / cell_len) + 1, ny = (int)((yed - yst) / cell_len) + 1;
  int nz = (int)((zed - zst) / cell_len) + 1;
  int id_level = 0;
  double maxD_lvl = maxD;
  for (int idh = 1; idh <= numLevels; idh++) {
    double minD_lvl = maxD_lvl / 2.0;
    if (idh == numLevels) minD_lvl = 0.0;
    int populated = 0;
    for (int t = 0; t < h->nT; t++) {
      double d = 2.0 * h->Radius[t];
      if (d > minD_lvl && (idh == 1 || d <= maxD_lvl)) populated = 1;
    }
    if (populated) {
      id_level++;
      for (int t = 0; t < h->nT; t++) {
        double d = 2.0 * h->Radius[t];
        if (d > minD_lvl && (idh == 1 || d <= maxD_lvl)) h->type_level[t] = id_level;
      }
      struct hlvl* L = &h->lvls[id_level];
      L->lvl = id_level;
      L->lvl_multiple = idh;
      L->nx = nx; L->ny = ny; L->nz = nz;
      L->cell_len = cell_len;
      L->HeadY = (int*)xcalloc((size_t)ny + 2, sizeof(int));
      L->HeadX0 = (int*)xcalloc((size_t)nx + 2, sizeof(int));
      L->HeadX = (int*)xcalloc((size_t)nx + 2, sizeof(int));
      L->HeadX2 = (int*)xcalloc((size_t)nx + 2, sizeof(int));
      L->HeadZ0 = (int*)xcalloc((size_t)3 * (nz + 2), sizeof(int));
      L->HeadZ = (int*)xcalloc((size_t)3 * (nz + 2), sizeof(int));
      L->HeadZ2 = (int*)xcalloc((size_t)3 * (nz + 2), sizeof(int));
      for (int i = 0; i < ny + 2; i++) L->HeadY[i] = -1;
      for (int i = 0; i < nx + 2; i++) L->HeadX0[i] = L->HeadX[i] = L->HeadX2[i] = -1;
      for (int i = 0; i < 3 * (nz + 2); i++) L->HeadZ0[i] = L->HeadZ[i] = L->HeadZ2[i] = -1;
      L->curr_xList_ind = -1;
      L->curr_xList2_ind = -1;
      for (int m = 0; m < 3; m++) L->curr_zList0_ind[m] = L->curr_zList_ind[m] = L->curr_zList2_ind[m] = -1;
    }
    nx *= 2; ny *= 2; nz *= 2;
    maxD_lvl = minD_lvl;
    cell_len = cell_len / 2.0;
  }
  h->num_lvls = id_level;
}

/* NBSMH_clcBoxIndex_and_BuildYList, :247-336 */
static int hbox_and_ylist(orc* h) {
  int n12 = h->nlocal + h->nGhost;
  if (n12 >= h->mbox) grow_nbs(h);
  for (int k = 1; k <= h->num_lvls; k++) {
    struct hlvl* L = &h->lvls[k];
    for (int i = 0; i < L->ny + 2; i++) L->HeadY[i] = -1;
  }
  for (int i = 1; i <= n12; i++) {
    r4 P;
    int t;
    if (i <= h->nlocal) { P = h->PosR[i]; t = h->pType[i]; }
    else { P = h->GhostP_PosR[i - h->nlocal]; t = h->GhostP_pType[i - h->nlocal]; }
    double rpdx = P.x - h->xst_cs, rpdy = P.y - h->yst_cs, rpdz = P.z - h->zst_cs;
    struct hlvl* L = &h->lvls[h->type_level[t - 1]];
    double cl = L->cell_len;
    h->bx[i] = (int)floor(rpdx / cl) + 1;
    int iy = (int)floor(rpdy / cl) + 1;
    h->by[i] = iy;
    h->bz[i] = (int)floor(rpdz / cl) + 1;
    if (h->bx[i] < 1 || h->bx[i] > L->nx || iy < 1 || iy > L->ny || h->bz[i] < 1 || h->bz[i] > L->nz)
      return fail(h, SDEM_E_GRID, "NBSMH_clcBoxIndex: particle outside the search grid");
    h->NextY[i] = L->HeadY[iy];
    L->HeadY[iy] = i;
  }
  return 0;
}

static void hbuild_xlist(orc* h, struct hlvl* L, int iy) { /* :341-361 */
  if (iy == L->curr_xList_ind) return;
  for (int i = 0; i < L->nx + 2; i++) L->HeadX[i] = -1;
  L->curr_xList_ind = iy;
  int n = L->HeadY[iy];
  while (n != -1) {
    int ix = h->bx[n];
    h->NextX[n] = L->HeadX[ix];
    L->HeadX[ix] = n;
    n = h->NextY[n];
  }
}

static void hbuild_xlist2(orc* h, struct hlvl* L, int iy) { /* :366-386 */
  if (iy == L->curr_xList2_ind) return;
  for (int i = 0; i < L->nx + 2; i++) L->HeadX2[i] = -1;
  L->curr_xList_ind = iy;   /* the reference records the row here (:380) */
  int n = L->HeadY[iy];
  while (n != -1) {
    int ix = h->bx[n];
    h->NextX[n] = L->HeadX2[ix];
    L->HeadX2[ix] = n;
    n = h->NextY[n];
  }
}

/* BuildZList0 / BuildZList / BuildZList2 (:391-475): column ix+m-1 of the
 * row below / this row / the row above */
static void hbuild_zl(orc* h, struct hlvl* L, int* head_x, int* head_z, int* curr, int ix, int m, int lcheck) {
  if (lcheck && ix == curr[m]) return;
  for (int iz = 0; iz < L->nz + 2; iz++) head_z[m * (L->nz + 2) + iz] = -1;
  curr[m] = ix;
  int n = head_x[ix + m - 1];
  while (n != -1) {
    int iz = h->bz[n];
    h->NextZ[n] = head_z[m * (L->nz + 2) + iz];
    head_z[m * (L->nz + 2) + iz] = n;
    n = h->NextX[n];
  }
}

/* NBSMH_FineSearch, :709-753 (pid1 the partner, pid2 the target) */
static void hfine_search(orc* h, int pid1, int pid2) {
  const int nl = h->nlocal;
  double dx, dy, dz, dr, d2sum, dr2, ovrlp;
  if (pid1 > nl || pid2 > nl) {
    const int gid = pid1 > nl ? pid1 - nl : pid2 - nl;
    const int loc = pid1 > nl ? pid2 : pid1;
    r4 A = pid1 > nl ? h->GhostP_PosR[gid] : h->PosR[pid1];
    r4 B = pid1 > nl ? h->PosR[pid2] : h->GhostP_PosR[gid];
    dr = A.w + B.w;
    dr2 = dr * dr;
    dx = A.x - B.x;
    d2sum = dx * dx;
    if (d2sum > dr2) return;
    dy = A.y - B.y;
    d2sum = dy * dy + d2sum;
    if (d2sum > dr2) return;
    dz = A.z - B.z;
    d2sum = dz * dz + d2sum;
    if (d2sum > dr2) return;
    ovrlp = dr - sqrt(d2sum);
    add_contact_ppg(h, loc, gid, ovrlp);
    return;
  }
  dr = h->PosR[pid1].w + h->PosR[pid2].w;
  dr2 = dr * dr;
  dx = h->PosR[pid1].x - h->PosR[pid2].x;
  d2sum = dx * dx;
  if (d2sum > dr2) return;
  dy = h->PosR[pid1].y - h->PosR[pid2].y;
  d2sum = dy * dy + d2sum;
  if (d2sum > dr2) return;
  dz = h->PosR[pid1].z - h->PosR[pid2].z;
  d2sum = dz * dz + d2sum;
  if (d2sum > dr2) return;
  ovrlp = dr - sqrt(d2sum);
  if (h->id[pid1] < h->id[pid2]) add_contact_pp(h, pid1, pid2, ovrlp);
  else add_contact_pp(h, pid2, pid1, ovrlp);
}

/* NBSMH_LoopNBSMask, :601-704 */
static void hloop_nbs_mask(orc* h, struct hlvl* L, int iz) {
  const int nl = h->nlocal;
  int m = HLZ(L, HeadZ, 1, iz);
  while (m != -1) {
    const int ghost = m > nl;
#define HVISIT(start) do { int n_ = (start); while (n_ != -1) { if (!ghost || n_ <= nl) { hfine_search(h, n_, m); h->num_Cnsv++; } n_ = h->NextZ[n_]; } } while (0)
    HVISIT(h->NextZ[m]);
    HVISIT(HLZ(L, HeadZ, 1, iz - 1));
    for (int i = -1; i <= 1; i++) HVISIT(HLZ(L, HeadZ, 0, iz + i));
    for (int lx = 0; lx <= 2; lx++)
      for (int i = -1; i <= 1; i++) HVISIT(HLZ(L, HeadZ0, lx, iz + i));
#undef HVISIT
    m = h->NextZ[m];
  }
}

/* NBSMH_Loop_CrossMask, :762-863: 27 cells of the coarser level (row below,
 * this row, row above; columns crs_ix-1..+1; cells crs_iz-1..+1) */
static void hloop_cross(orc* h, struct hlvl* L, int iz, int crs_iz, struct hlvl* X) {
  const int nl = h->nlocal;
  int m = HLZ(L, HeadZ, 1, iz);
  while (m != -1) {
    const int ghost = m > nl;
#define XVISIT(start) do { int n_ = (start); while (n_ != -1) { if (!ghost || n_ <= nl) { hfine_search(h, n_, m); h->lvl_num_cnsv++; } n_ = h->NextZ[n_]; } } while (0)
    for (int lx = 0; lx <= 2; lx++)
      for (int l = -1; l <= 1; l++) XVISIT(HLZ(X, HeadZ0, lx, crs_iz + l));
    for (int lx = 0; lx <= 2; lx++)
      for (int l = -1; l <= 1; l++) XVISIT(HLZ(X, HeadZ, lx, crs_iz + l));
    for (int lx = 0; lx <= 2; lx++)
      for (int l = -1; l <= 1; l++) XVISIT(HLZ(X, HeadZ2, lx, crs_iz + l));
#undef XVISIT
    m = h->NextZ[m];
  }
}

static void hcopy(int* dst, const int* src, int n) { memcpy(dst, src, sizeof(int) * (size_t)n); }

/* OneLevelBroadSearch, :480-596 */
static void one_level(orc* h, struct hlvl* B) {
  const int zs = B->nz + 2;
  for (int i = 0; i < B->nx + 2; i++) B->HeadX0[i] = -1;
  for (int iy = 1; iy <= B->ny; iy++) {
    hbuild_xlist(h, B, iy);
    for (int idh = B->lvl - 1; idh >= 1; idh--) {
      struct hlvl* X = &h->lvls[idh];
      int coe = 1 << (B->lvl_multiple - X->lvl_multiple);
      int crs_y = (iy - 1) / coe + 1;
      if (crs_y == 1) {
        for (int i = 0; i < X->nx + 2; i++) X->HeadX0[i] = -1;
        hbuild_xlist(h, X, 1);
      }
      hbuild_xlist2(h, X, crs_y + 1);
    }
    if (B->HeadY[iy] != -1) {
      for (int iz = 0; iz < zs; iz++) { HLZ(B, HeadZ, 0, iz) = -1; HLZ(B, HeadZ0, 0, iz) = -1; }
      hbuild_zl(h, B, B->HeadX0, B->HeadZ0, B->curr_zList0_ind, 1, 1, 0);
      for (int ix = 1; ix <= B->nx; ix++) {
        hbuild_zl(h, B, B->HeadX, B->HeadZ, B->curr_zList_ind, ix, 1, 0);
        hbuild_zl(h, B, B->HeadX0, B->HeadZ0, B->curr_zList0_ind, ix, 2, 0);
        for (int idh = B->lvl - 1; idh >= 1; idh--) {
          struct hlvl* X = &h->lvls[idh];
          int coe = 1 << (B->lvl_multiple - X->lvl_multiple);
          int crs_x = (ix - 1) / coe + 1;
          const int xzs = X->nz + 2;
          if (crs_x == 1) {
            for (int iz = 0; iz < xzs; iz++) { HLZ(X, HeadZ0, 0, iz) = -1; HLZ(X, HeadZ, 0, iz) = -1; HLZ(X, HeadZ2, 0, iz) = -1; }
            hbuild_zl(h, X, X->HeadX0, X->HeadZ0, X->curr_zList0_ind, crs_x, 1, 1);
            hbuild_zl(h, X, X->HeadX, X->HeadZ, X->curr_zList_ind, crs_x, 1, 1);
            hbuild_zl(h, X, X->HeadX2, X->HeadZ2, X->curr_zList2_ind, crs_x, 1, 1);
          }
          hbuild_zl(h, X, X->HeadX0, X->HeadZ0, X->curr_zList0_ind, crs_x, 2, 1);
          hbuild_zl(h, X, X->HeadX, X->HeadZ, X->curr_zList_ind, crs_x, 2, 1);
          hbuild_zl(h, X, X->HeadX2, X->HeadZ2, X->curr_zList2_ind, crs_x, 2, 1);
        }
        if (B->HeadX[ix] != -1) {
          for (int iz = 1; iz <= B->nz; iz++) {
            hloop_nbs_mask(h, B, iz);
            for (int idh = B->lvl - 1; idh >= 1; idh--) {
              struct hlvl* X = &h->lvls[idh];
              int coe = 1 << (B->lvl_multiple - X->lvl_multiple);
              hloop_cross(h, B, iz, (iz - 1) / coe + 1, X);
            }
          }
        }
        hcopy(&HLZ(B, HeadZ, 0, 0), &HLZ(B, HeadZ, 1, 0), zs);
        hcopy(&HLZ(B, HeadZ0, 0, 0), &HLZ(B, HeadZ0, 1, 0), zs);
        hcopy(&HLZ(B, HeadZ0, 1, 0), &HLZ(B, HeadZ0, 2, 0), zs);
        for (int idh = B->lvl - 1; idh >= 1; idh--) {
          struct hlvl* X = &h->lvls[idh];
          int coe = 1 << (B->lvl_multiple - X->lvl_multiple);
          if (ix % coe == 0) {
            const int xzs = X->nz + 2;
            hcopy(&HLZ(X, HeadZ0, 0, 0), &HLZ(X, HeadZ0, 1, 0), xzs);
            hcopy(&HLZ(X, HeadZ0, 1, 0), &HLZ(X, HeadZ0, 2, 0), xzs);
            X->curr_zList0_ind[0] = X->curr_zList0_ind[1];
            X->curr_zList0_ind[1] = X->curr_zList0_ind[2];
            hcopy(&HLZ(X, HeadZ, 0, 0), &HLZ(X, HeadZ, 1, 0), xzs);
            hcopy(&HLZ(X, HeadZ, 1, 0), &HLZ(X, HeadZ, 2, 0), xzs);
            X->curr_zList_ind[0] = X->curr_zList_ind[1];
            X->curr_zList_ind[1] = X->curr_zList_ind[2];
            hcopy(&HLZ(X, HeadZ2, 0, 0), &HLZ(X, HeadZ2, 1, 0), xzs);
            hcopy(&HLZ(X, HeadZ2, 1, 0), &HLZ(X, HeadZ2, 2, 0), xzs);
            X->curr_zList2_ind[0] = X->curr_zList2_ind[1];
            X->curr_zList2_ind[1] = X->curr_zList2_ind[2];
          }
        }
        if (h->err) return;
      }
    }
    hcopy(B->HeadX0, B->HeadX, B->nx + 2);
    for (int idh = B->lvl - 1; idh >= 1; idh--) {
      struct hlvl* X = &h->lvls[idh];
      int coe = 1 << (B->lvl_multiple - X->lvl_multiple);
      if (iy % coe == 0) {
        hcopy(X->HeadX0, X->HeadX, X->nx + 2);
        hcopy(X->HeadX, X->HeadX2, X->nx + 2);
        X->curr_xList_ind = X->curr_xList2_ind;
      }
    }
  }
}

/* NBSMH_ContactSearch, :227-242 */
static int nbsmh_contact_search(orc* h) {
  h->num_Cnsv = 0;
  h->lvl_num_cnsv = 0;
  if (h->nlocal == 0) return 0;
  if (hbox_and_ylist(h)) return h->err;
  for (int idh = h->num_lvls; idh >= 1; idh--) {
    one_level(h, &h->lvls[idh]);
    if (h->err) return h->err;
  }
  return 0;
}

/* ---- plane walls (Prtcl_Geometry.f90) ---------------------------------- */
static int pw_is_in_plane(r3 p1, r3 p2, r3 p3, r3 p4, r3 cp) { /* :185-221 */
  r3 p1p = r3sub(p1, cp), p2p = r3sub(p2, cp), p3p = r3sub(p3, cp), p4p = r3sub(p4, cp);
  double p1p3 = r3dot(p1p, p3p), p2p4 = r3dot(p2p, p4p), p1p4 = r3dot(p1p, p4p), p2p3 = r3dot(p2p, p3p);
  if (p1p3 * p2p4 - p1p4 * p2p3 < 0.0) return 0;
  double p1p2 = r3dot(p1p, p2p), p3p4 = r3dot(p3p, p4p);
  if (p1p3 * p2p4 - p1p2 * p3p4 < 0.0) return 0;
  double p2p2 = r3dot(p2p, p2p);
  if (p1p2 * p2p3 - p1p3 * p2p2 < 0.0) return 0;
  return 1;
}

static int line_point_check(r3 lp1, r3 lp2, r4 dpos, r3* nv, double* ovrlp) { /* :226-261 */
  r3 pos = r4xyz(dpos), cp;
  r3 w = r3sub(pos, lp1);
  r3 v = r3sub(lp2, lp1);
  double length = r3norm(r3sub(lp1, lp2));
  double r = dpos.w;
  double t = r3dot(w, v) / r3dot(v, v);
  if (t >= 0.0 && t <= 1.0) cp = r3add(r3scale(v, t), lp1);
  else if (t >= (-r / length) && t < 0.0) cp = lp1;
  else if (t > 1.0 && t >= (1.0 + r / length)) cp = lp2;
  else return 0;
  *ovrlp = r - r3norm(r3sub(cp, pos));
  if (*ovrlp >= 0.0) {
    *nv = nv_of(r3sub(pos, cp));
    return 1;
  }
  return 0;
}

static int pw_is_in_contact(const wall_t* W, r4 box, double* ovrlp, r3* nv) { /* :55-109 */
  double Radius = box.w, dist, t;
  r3 p = r4xyz(box), cp;
  dist = r3dot(W->n, p) + W->d;
  if (W->bothSide) {
    *ovrlp = Radius - fabs(dist);
  } else {
    if (dist < 0.0) return 0;
    *ovrlp = Radius - dist;
  }
  if (*ovrlp < 0.0) return 0;
  if (W->isInfinite) {
    *nv = r3scale(W->n, copysign(1.0, dist));
    return 1;
  }
  t = -dist;
  cp = r3add(r3scale(W->n, t), p);
  if (pw_is_in_plane(W->p1, W->p2, W->p3, W->p4, cp)) {
    *nv = r3scale(W->n, copysign(1.0, dist));
    return 1;
  }
  if (line_point_check(W->p1, W->p2, box, nv, ovrlp)) return 1;
  if (line_point_check(W->p2, W->p3, box, nv, ovrlp)) return 1;
  if (line_point_check(W->p3, W->p4, box, nv, ovrlp)) return 1;
  if (line_point_check(W->p4, W->p1, box, nv, ovrlp)) return 1;
  return 0;
}

/* UpdateNearPrtclsPW, Prtcl_ContactSearchPW.f90:159-235 */
static void update_near_prtcls_pw(orc* h, int iterNumber) {
  if (iterNumber < h->Next_iter_update) return;
  init_pwcs_list(h);
  for (int wid = 1; wid <= h->nw; wid++) {
    const wall_t* W = &h->walls[wid - 1];
    r3 pmin = r3sub(W->min_point, (r3){h->DeltaXmax2, h->DeltaXmax2, h->DeltaXmax2});
    r3 pmax = r3add(W->max_point, (r3){h->DeltaXmax2, h->DeltaXmax2, h->DeltaXmax2});
    for (int i = 1; i <= h->nlocal; i++) {
      r4 P = h->PosR[i];
      if (P.x >= pmin.x && P.x <= pmax.x && P.y >= pmin.y && P.y <= pmax.y && P.z >= pmin.z &&
          P.z <= pmax.z) {
        if (h->NextInsertPW == 0) realloc_pwcs_list(h);
        int nextI = h->NextInsertPW;
        h->NextInsertPW = -h->Next_PWCS[nextI];
        h->id_Wall[nextI] = wid;
        h->Next_PWCS[nextI] = h->Bucket_PWCS[i];
        h->Bucket_PWCS[i] = nextI;
      }
    }
  }
  double maxreal = 0.0, max_v, max_a, t;
  for (int i = 1; i <= h->nlocal; i++) {
    double v = r3norm(LV(h, 1, i));
    maxreal = (maxreal > v) ? maxreal : v;
  }
  max_v = maxreal + h->MaxWallVel;
  max_v = (max_v > 0.3) ? max_v : 0.3;
  max_v = max_v * 1.5;
  maxreal = 0.0;
  for (int i = 1; i <= h->nlocal; i++) {
    double a = r3norm(LA(h, 1, i));
    maxreal = (maxreal > a) ? maxreal : a;
  }
  double g = r3norm((r3){h->cfg.gravity[0], h->cfg.gravity[1], h->cfg.gravity[2]});
  max_a = (maxreal > g) ? maxreal : g;
  max_a = max_a * 1.5;
  t = (sqrt(max_v * max_v + 2.0 * max_a * h->DeltaXmax1) - max_v) / max_a;
  int numIter = (int)(t / h->cfg.dt);
  numIter = numIter > 1 ? numIter : 1;
  numIter = numIter < h->cfg.wall_max_update_iter ? numIter : h->cfg.wall_max_update_iter;
  h->Next_iter_update = iterNumber + numIter;
}

/* FindContactsPW, Prtcl_ContactSearchPW.f90:298-319 */
static void find_contacts_pw(orc* h) {
  for (int i = 1; i <= h->nlocal; i++) {
    int nid = h->Bucket_PWCS[i];
    while (nid > 0) {
      int wid = h->id_Wall[nid];
      double ovrlp;
      r3 nv;
      if (pw_is_in_contact(&h->walls[wid - 1], h->PosR[i], &ovrlp, &nv))
        add_contact_pw(h, i, wid, ovrlp, nv);
      nid = h->Next_PWCS[nid];
    }
  }
}

/* ---- acceleration + integration --------------------------------------- */
static void clc_acceleration(orc* h) { /* Prtcl_DEMSystem.f90:166-181 */
  r3 g = {h->cfg.gravity[0], h->cfg.gravity[1], h->cfg.gravity[2]};
  for (int i = 1; i <= h->nlocal; i++) {
    int it = h->pType[i];
    double Mass = h->Mass[it - 1], Inertia = h->Inertia[it - 1];
    LA(h, 1, i) = r3add(r3div(h->F[i], Mass), g);
    RA(h, 1, i) = r3div(h->T[i], Inertia);
  }
}

static void prtcl_integrate(orc* h) { /* Prtcl_Integration.f90:15-88 */
  const double AB2C1 = 3.0 / 2.0, AB2C2 = -1.0 / 2.0;
  const double AB3C1 = 23.0 / 12.0, AB3C2 = -16.0 / 12.0, AB3C3 = 5.0 / 12.0;
  double dt = h->cfg.dt;
  int n = h->nlocal;
#define ADDPOS(P, v) do { (P).x = (P).x + (v).x; (P).y = (P).y + (v).y; (P).z = (P).z + (v).z; } while (0)
  if (h->cfg.pi_method == SDEM_PIM_FE) {
    for (int i = 1; i <= n; i++) {
      r3 s = r3scale(LV(h, 1, i), dt);
      ADDPOS(h->PosR[i], s);
      LV(h, 1, i) = r3add(LV(h, 1, i), r3scale(LA(h, 1, i), dt));
    }
  } else if (h->cfg.pi_method == SDEM_PIM_AB2) {
    for (int i = 1; i <= n; i++) {
      r3 v1 = LV(h, 1, i);
      r3 s = r3scale(r3add(r3scale(v1, AB2C1), r3scale(LV(h, 2, i), AB2C2)), dt);
      ADDPOS(h->PosR[i], s);
      LV(h, 1, i) = r3add(v1, r3scale(r3add(r3scale(LA(h, 1, i), AB2C1), r3scale(LA(h, 2, i), AB2C2)), dt));
      LV(h, 2, i) = v1;
      LA(h, 2, i) = LA(h, 1, i);
    }
  } else if (h->cfg.pi_method == SDEM_PIM_AB3) {
    for (int i = 1; i <= n; i++) {
      r3 v1 = LV(h, 1, i), v2 = LV(h, 2, i);
      r3 s = r3scale(r3add(r3add(r3scale(v1, AB3C1), r3scale(v2, AB3C2)), r3scale(LV(h, 3, i), AB3C3)), dt);
      ADDPOS(h->PosR[i], s);
      LV(h, 1, i) = r3add(v1, r3scale(r3add(r3add(r3scale(LA(h, 1, i), AB3C1), r3scale(LA(h, 2, i), AB3C2)),
                                            r3scale(LA(h, 3, i), AB3C3)), dt));
      LV(h, 3, i) = v2;
      LV(h, 2, i) = v1;
      LA(h, 3, i) = LA(h, 2, i);
      LA(h, 2, i) = LA(h, 1, i);
    }
  }
#undef ADDPOS
  if (h->cfg.pri_method == SDEM_PIM_FE) {
    for (int i = 1; i <= n; i++) {
      h->theta[i] = r3add(h->theta[i], r3scale(RV(h, 1, i), dt));
      RV(h, 1, i) = r3add(RV(h, 1, i), r3scale(RA(h, 1, i), dt));
    }
  } else if (h->cfg.pri_method == SDEM_PIM_AB2) {
    for (int i = 1; i <= n; i++) {
      /* Prtcl_Integration.f90:64 reads GPrtcl_linVel(1,i) here (quirk Q1). */
      r3 w1 = h->cfg.quirk_ab2_rot ? LV(h, 1, i) : RV(h, 1, i);
      h->theta[i] = r3add(h->theta[i], r3scale(r3add(r3scale(w1, AB2C1), r3scale(RV(h, 2, i), AB2C2)), dt));
      RV(h, 1, i) = r3add(w1, r3scale(r3add(r3scale(RA(h, 1, i), AB2C1), r3scale(RA(h, 2, i), AB2C2)), dt));
      RV(h, 2, i) = w1;
      RA(h, 2, i) = RA(h, 1, i);
    }
  } else if (h->cfg.pri_method == SDEM_PIM_AB3) {
    for (int i = 1; i <= n; i++) {
      r3 w1 = RV(h, 1, i), w2 = RV(h, 2, i);
      h->theta[i] = r3add(h->theta[i], r3scale(r3add(r3add(r3scale(w1, AB3C1), r3scale(w2, AB3C2)),
                                                     r3scale(RV(h, 3, i), AB3C3)), dt));
      RV(h, 1, i) = r3add(w1, r3scale(r3add(r3add(r3scale(RA(h, 1, i), AB3C1), r3scale(RA(h, 2, i), AB3C2)),
                                            r3scale(RA(h, 3, i), AB3C3)), dt));
      RV(h, 3, i) = w2;
      RV(h, 2, i) = w1;
      RA(h, 3, i) = RA(h, 2, i);
      RA(h, 2, i) = RA(h, 1, i);
    }
  }
}

/* ---- one-rank out-of-domain delete (y pencil, no periodicity) ---------- */
static void gl_copy(orc* h, int i1, int i2) { /* Prtcl_Variables.f90:351-373 */
  if (i1 == i2) return;
  h->id[i1] = h->id[i2];
  h->pType[i1] = h->pType[i2];
  h->usrMark[i1] = h->usrMark[i2];
  h->PosR[i1] = h->PosR[i2];
  for (int k = 1; k <= h->tsize; k++) { LV(h, k, i1) = LV(h, k, i2); LA(h, k, i1) = LA(h, k, i2); }
  h->theta[i1] = h->theta[i2];
  for (int k = 1; k <= h->rsize; k++) { RV(h, k, i1) = RV(h, k, i2); RA(h, k, i1) = RA(h, k, i2); }
  /* force/torque are not part of GL_copy */
}
static void cl_copy(orc* h, int id1, int id2) { /* Prtcl_CL_and_CF.f90:449-458 */
  h->Bucket[id1] = h->Bucket[id2];
  h->Head_Cp[id1] = h->Head_Cp[id2];
  h->Bucket[id2] = 0;
  h->Head_Cp[id2] = -1;
}
static void cspw_copy(orc* h, int id1, int id2) { /* Prtcl_ContactSearchPW.f90:240-259 */
  int n = h->Bucket_PWCS[id1];
  while (n > 0) {
    int NextI = h->Next_PWCS[n];
    h->Next_PWCS[n] = -h->NextInsertPW;
    h->NextInsertPW = n;
    n = NextI;
  }
  h->Bucket_PWCS[id1] = h->Bucket_PWCS[id2];
  h->Bucket_PWCS[id2] = 0;
}

static int out_of(orc* h, int i, int pass) {
  r4 P = h->PosR[i];
  const double* mn = h->cfg.dom_min;
  const double* mx = h->cfg.dom_max;
  switch (pass) {
    case 0: return P.y >= mx[1] || P.y < mn[1];
    case 1: return P.x >= mx[0];
    case 2: return P.x < mn[0];
    case 3: return P.z >= mx[2];
    default: return P.z < mn[2];
  }
}

/* PC_Comm_For_Exchange, y-pencil branch (Prtcl_Comm.f90:1569-1840) with one
 * rank: five passes (y, +x, -x, +z, -z); a periodic direction wraps the
 * positions (:1575-1582, :1612-1618, :1672-1678, ...), any other deletes the
 * particles outside [min, max) by swap-with-last. */
static void comm_for_exchange(orc* h) {
  int nlocal = h->nlocal;
  const double* mn = h->cfg.dom_min;
  const double* mx = h->cfg.dom_max;
  for (int pass = 0; pass < 5; pass++) {
    int dir = pass == 0 ? 1 : (pass <= 2 ? 0 : 2);
    if (h->cfg.periodic[dir]) {
      double Lk = mx[dir] - mn[dir];
      for (int i = 1; i <= nlocal; i++) {
        double* c = dir == 0 ? &h->PosR[i].x : (dir == 1 ? &h->PosR[i].y : &h->PosR[i].z);
        double v = *c;
        if (pass == 0) {
          if (v >= mx[1]) *c = v - Lk;
          else if (v < mn[1]) *c = v + Lk;
        } else if (pass == 1 || pass == 3) {
          if (v >= mx[dir]) *c = v - Lk;
        } else {
          if (v < mn[dir]) *c = v + Lk;
        }
      }
      continue;
    }
    int i = 1;
    while (i <= nlocal) {
      if (out_of(h, i, pass)) {
        gl_copy(h, i, nlocal);
        cl_copy(h, i, nlocal);
        cspw_copy(h, i, nlocal);
        nlocal = nlocal - 1;
      } else {
        i = i + 1;
      }
    }
  }
  h->nlocal = nlocal;
}

/* ---- one time step (DEMS_iterate, Prtcl_DEMSystem.f90:201-252) --------- */
int orc_step(orc* h, int nsteps) {
  if (!h->have_types) return fail(h, SDEM_E_ARG, "orc_step: tables not set");
  for (int s = 0; s < nsteps; s++) {
    /* DEMS_preIteration :322-331 */
    update_near_prtcls_pw(h, h->iterNumber);
    for (int i = 1; i <= h->nlocal; i++) { h->F[i] = zero_r3; h->T[i] = zero_r3; }
    cl_pre_iteration(h);
    comm_for_cntct(h);
    if ((h->cfg.cs_method == SDEM_CSM_HRCHL ? nbsmh_contact_search(h) : nbsm_contact_search(h))) return h->err;
    find_contacts_pw(h);
    if (h->err) return h->err;
    clc_acceleration(h);
    prtcl_integrate(h);
    comm_for_exchange(h);
    cl_remv_released(h);
    h->iterNumber++;
  }
  return 0;
}

void orc_set_iter(orc* h, int iterNumber) { h->iterNumber = iterNumber; }

/* ---- downloads ----------------------------------------------------------- */
int orc_nlocal(orc* h) { return h->nlocal; }

int orc_download_particles(orc* h, int* id, int* ptype, int* usrmark, double* posR,
                           double* linVel, double* linAcc, double* theta,
                           double* rotVel, double* rotAcc) {
  int ts = h->tsize, rs = h->rsize;
  for (int i = 1; i <= h->nlocal; i++) {
    int q = i - 1;
    if (id) id[q] = h->id[i];
    if (ptype) ptype[q] = h->pType[i];
    if (usrmark) usrmark[q] = h->usrMark[i];
    if (posR) { posR[4 * q] = h->PosR[i].x; posR[4 * q + 1] = h->PosR[i].y; posR[4 * q + 2] = h->PosR[i].z; posR[4 * q + 3] = h->PosR[i].w; }
    for (int k = 1; k <= ts; k++) {
      if (linVel) { double* v = linVel + ((size_t)q * ts + k - 1) * 3; v[0] = LV(h, k, i).x; v[1] = LV(h, k, i).y; v[2] = LV(h, k, i).z; }
      if (linAcc) { double* v = linAcc + ((size_t)q * ts + k - 1) * 3; v[0] = LA(h, k, i).x; v[1] = LA(h, k, i).y; v[2] = LA(h, k, i).z; }
    }
    for (int k = 1; k <= rs; k++) {
      if (rotVel) { double* v = rotVel + ((size_t)q * rs + k - 1) * 3; v[0] = RV(h, k, i).x; v[1] = RV(h, k, i).y; v[2] = RV(h, k, i).z; }
      if (rotAcc) { double* v = rotAcc + ((size_t)q * rs + k - 1) * 3; v[0] = RA(h, k, i).x; v[1] = RA(h, k, i).y; v[2] = RA(h, k, i).z; }
    }
    if (theta) { theta[3 * q] = h->theta[i].x; theta[3 * q + 1] = h->theta[i].y; theta[3 * q + 2] = h->theta[i].z; }
  }
  return 0;
}

int orc_download_forces(orc* h, double* F, double* T) {
  for (int i = 1; i <= h->nlocal; i++) {
    int q = i - 1;
    if (F) { F[3 * q] = h->F[i].x; F[3 * q + 1] = h->F[i].y; F[3 * q + 2] = h->F[i].z; }
    if (T) { T[3 * q] = h->T[i].x; T[3 * q + 1] = h->T[i].y; T[3 * q + 2] = h->T[i].z; }
  }
  return 0;
}

/* Every live contact as the restart writer lists it (CL_Gather_Cntctlink_Restart,
 * Prtcl_CL_and_CF.f90:656-685): bucket entries then Head_Cp entries per particle.
 * With cap < count, only *nc is set. */
int orc_download_contacts(orc* h, int cap, int* nc, int* owner_idx, int* partner_id,
                          double* tandelta, double* velrel) {
  int c = 0;
  for (int pass = 0; pass < 2; pass++) {
    c = 0;
    for (int pid = 1; pid <= h->nlocal; pid++) {
      int n = h->Bucket[pid];
      while (n > 0) {
        if (pass) {
          owner_idx[c] = pid - 1; partner_id[c] = h->id_j[n];
          tandelta[3 * c] = h->TanDelta[n].x; tandelta[3 * c + 1] = h->TanDelta[n].y; tandelta[3 * c + 2] = h->TanDelta[n].z;
          velrel[c] = h->VelRel_Init[n];
        }
        c++;
        n = h->Next[n];
      }
      n = h->Head_Cp[pid];
      while (n != -1) {
        if (pass) {
          owner_idx[c] = pid - 1; partner_id[c] = h->id_i[n];
          tandelta[3 * c] = h->TanDelta[n].x; tandelta[3 * c + 1] = h->TanDelta[n].y; tandelta[3 * c + 2] = h->TanDelta[n].z;
          velrel[c] = h->VelRel_Init[n];
        }
        c++;
        n = h->Next_Cp[n];
      }
    }
    *nc = c;
    if (c > cap || !owner_idx) return 0;
  }
  return 0;
}

int orc_counters(orc* h, int* out) {
  out[SDEM_CNT_PP] = h->numCntcts[0];
  out[SDEM_CNT_PPG] = h->numCntcts[1];
  out[SDEM_CNT_PPFIX] = h->numCntcts[2];
  out[SDEM_CNT_PW] = h->numCntcts[3];
  out[SDEM_CNT_CNSV] = (int)h->num_Cnsv;
  out[SDEM_CNT_NLOCAL] = h->nlocal;
  out[SDEM_CNT_ITER] = h->iterNumber;
  out[SDEM_CNT_NEXTWALL] = h->Next_iter_update;
  out[SDEM_CNT_CNSV_CROSS] = (int)h->lvl_num_cnsv;
  return 0;
}

/* grid geometry of the search (for tests of the binning) */
void orc_grid(orc* h, double* cell_len, double* origin, int* dims) {
  *cell_len = h->cell_len;
  origin[0] = h->xst_cs; origin[1] = h->yst_cs; origin[2] = h->zst_cs;
  dims[0] = h->nx; dims[1] = h->ny; dims[2] = h->nz;
}

void orc_destroy(orc* h) {
  if (!h) return;
  free(h->FixId); free(h->FixType); free(h->FixPosR);
  for (int k = 1; k <= h->num_lvls; k++) hlvl_free(&h->lvls[k]);
  free(h->lvls); free(h->type_level);
  free(h->id); free(h->pType); free(h->usrMark); free(h->PosR);
  free(h->linVel); free(h->linAcc); free(h->rotVel); free(h->rotAcc);
  free(h->theta); free(h->F); free(h->T);
  free(h->Bucket); free(h->id_j); free(h->Next); free(h->CntctStatus);
  free(h->TanDelta); free(h->VelRel_Init); free(h->id_i); free(h->Head_Cp); free(h->Next_Cp);
  free(h->bx); free(h->by); free(h->bz); free(h->NextX); free(h->NextY); free(h->NextZ);
  free(h->HeadY); free(h->HeadX); free(h->HeadX0); free(h->HeadZ); free(h->HeadZ0);
  free(h->Bucket_PWCS); free(h->id_Wall); free(h->Next_PWCS);
  free(h->Radius); free(h->Mass); free(h->Inertia); free(h->bpp); free(h->bpw);
  free(h->walls);
  free(h->GhostP_id); free(h->GhostP_pType); free(h->GhostP_PosR); free(h->GhostP_linVel); free(h->GhostP_rotVel);
  free(h);
}
