// dem_device.cuh -- device-side vector algebra, plane-wall geometry and the
// contact force law of sDEM, in the reference's exact order of floating-point
// operations.  The translation unit that includes this file is compiled with
// -fmad=false, so no a*b+c below is contracted into an FMA: every result is
// the IEEE-rounded value of the reference's expression (gfortran, x86-64,
// default flags).  Division and sqrt are correctly rounded; they run on the
// integer pipes (fp64_int.cuh), which GB300 has in plenty while its FP64 pipe
// bounds the force law, and give the IEEE results bit for bit.
#pragma once
#include <cuda_runtime.h>
#include "../../include/sdem_gpu.h"
#include "fp64_int.cuh"

namespace sdem {

// 32-byte aligned (x, y, z, w): one L2 sector per particle gather.
typedef double4_32a dbl4;
__host__ __device__ __forceinline__ dbl4 make_dbl4(double x, double y, double z, double w) {
  dbl4 r;
  r.x = x;
  r.y = y;
  r.z = z;
  r.w = w;
  return r;
}

struct r3 {
  double x, y, z;
};

__device__ __forceinline__ r3 mk3(double x, double y, double z) {
  r3 r;
  r.x = x;
  r.y = y;
  r.z = z;
  return r;
}
__device__ __forceinline__ r3 xyz(const dbl4& a) { return mk3(a.x, a.y, a.z); }
__device__ __forceinline__ dbl4 d4(r3 a, double w) { return make_dbl4(a.x, a.y, a.z, w); }

// Prtcl_TypeDef.f90 operators (:105-288)
__device__ __forceinline__ r3 add3(r3 a, r3 b) { return mk3(a.x + b.x, a.y + b.y, a.z + b.z); }
__device__ __forceinline__ r3 sub3(r3 a, r3 b) { return mk3(a.x - b.x, a.y - b.y, a.z - b.z); }
__device__ __forceinline__ r3 scale3(r3 p, double v) { return mk3(p.x * v, p.y * v, p.z * v); }
__device__ __forceinline__ r3 div3(r3 p, double v) {
  const fpi::Divisor dv = fpi::divisor(v);   // one reciprocal refinement for three quotients
  return mk3(fpi::div_by(p.x, dv), fpi::div_by(p.y, dv), fpi::div_by(p.z, dv));
}
__device__ __forceinline__ double dot3(r3 a, r3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
__device__ __forceinline__ r3 cross3(r3 u, r3 v) {
  return mk3(u.y * v.z - u.z * v.y, u.z * v.x - u.x * v.z, u.x * v.y - u.y * v.x);
}
__device__ __forceinline__ double norm3(r3 p) { return fpi::sqrt_rn(p.x * p.x + p.y * p.y + p.z * p.z); }
// real4_nv / real3_nv: s/|s| with the 1e-10 guard
__device__ __forceinline__ r3 nv3(r3 s) {
  double n = norm3(s);
  if (fpi::gt(n, 1.0000E-10)) return div3(s, n);
  return mk3(0.0, 0.0, 0.0);
}

// One plane wall as uploaded (SDEM_W_* layout).
struct Wall {
  r3 p1, p2, p3, p4, n, vel, mn, mx;
  double d;
  int bothSide, isInfinite, wall_id, wall_type;
};

__device__ __forceinline__ Wall load_wall(const double* w, const int* f, int k) {
  const double* r = w + k * SDEM_W_SIZE;
  Wall W;
  W.p1 = mk3(r[0], r[1], r[2]);
  W.p2 = mk3(r[3], r[4], r[5]);
  W.p3 = mk3(r[6], r[7], r[8]);
  W.p4 = mk3(r[9], r[10], r[11]);
  W.n = mk3(r[12], r[13], r[14]);
  W.d = r[15];
  W.vel = mk3(r[16], r[17], r[18]);
  W.mn = mk3(r[19], r[20], r[21]);
  W.mx = mk3(r[22], r[23], r[24]);
  const int* q = f + k * SDEM_WF_SIZE;
  W.bothSide = q[0];
  W.isInfinite = q[1];
  W.wall_id = q[2];
  W.wall_type = q[3];
  return W;
}

// PW_IsInPlane, Prtcl_Geometry.f90:185-221
__device__ __forceinline__ bool in_plane(r3 p1, r3 p2, r3 p3, r3 p4, r3 cp) {
  r3 p1p = sub3(p1, cp), p2p = sub3(p2, cp), p3p = sub3(p3, cp), p4p = sub3(p4, cp);
  double p1p3 = dot3(p1p, p3p), p2p4 = dot3(p2p, p4p), p1p4 = dot3(p1p, p4p), p2p3 = dot3(p2p, p3p);
  if (p1p3 * p2p4 - p1p4 * p2p3 < 0.0) return false;
  double p1p2 = dot3(p1p, p2p), p3p4 = dot3(p3p, p4p);
  if (p1p3 * p2p4 - p1p2 * p3p4 < 0.0) return false;
  double p2p2 = dot3(p2p, p2p);
  if (p1p2 * p2p3 - p1p3 * p2p2 < 0.0) return false;
  return true;
}

// Line_point_check, Prtcl_Geometry.f90:226-261
__device__ __forceinline__ bool line_point(r3 lp1, r3 lp2, dbl4 dpos, r3& nv, double& ovrlp) {
  r3 pos = xyz(dpos), cp;
  r3 w = sub3(pos, lp1);
  r3 v = sub3(lp2, lp1);
  double length = norm3(sub3(lp1, lp2));
  double r = dpos.w;
  double t = fpi::div_rn(dot3(w, v), dot3(v, v));
  if (t >= 0.0 && t <= 1.0) cp = add3(scale3(v, t), lp1);
  else if (t >= fpi::div_rn(-r, length) && t < 0.0) cp = lp1;
  else if (t > 1.0 && t >= (1.0 + fpi::div_rn(r, length))) cp = lp2;
  else return false;
  ovrlp = r - norm3(sub3(cp, pos));
  if (ovrlp >= 0.0) {
    nv = nv3(sub3(pos, cp));
    return true;
  }
  return false;
}

// PW_isInContact, Prtcl_Geometry.f90:55-109
__device__ __forceinline__ bool wall_contact(const Wall& W, dbl4 box, double& ovrlp, r3& nv) {
  double Radius = box.w;
  r3 p = xyz(box);
  double dist = dot3(W.n, p) + W.d;
  if (W.bothSide) {
    ovrlp = Radius - fabs(dist);
  } else {
    if (dist < 0.0) return false;
    ovrlp = Radius - dist;
  }
  if (ovrlp < 0.0) return false;
  if (W.isInfinite) {
    nv = scale3(W.n, copysign(1.0, dist));
    return true;
  }
  double t = -dist;
  r3 cp = add3(scale3(W.n, t), p);
  if (in_plane(W.p1, W.p2, W.p3, W.p4, cp)) {
    nv = scale3(W.n, copysign(1.0, dist));
    return true;
  }
  if (line_point(W.p1, W.p2, box, nv, ovrlp)) return true;
  if (line_point(W.p2, W.p3, box, nv, ovrlp)) return true;
  if (line_point(W.p3, W.p4, box, nv, ovrlp)) return true;
  if (line_point(W.p4, W.p1, box, nv, ovrlp)) return true;
  return false;
}

// Force-law options fixed per handle.
struct LawCfg {
  int cf_type;   // SDEM_CFT_*
  int ct_model;  // SDEM_CTM_*
  double dt;
};

// The contact force law of Prtcl_ContactForce_inc.f90:1-66, shared by the
// particle-particle (ContactForce_PP, Prtcl_CL_and_CF.f90:732-756) and
// particle-wall (ContactForce_PW, :832-856) wrappers.
//   hist: in = (TanDelta, VelRel_Init) found for this pair, or (0,0,0,-2) for a
//         new contact (Find_insert, Prtcl_CL_and_CF.f90:293-294); out = updated.
//   S = Fnij + Ftij, M = Norm_v x Ftij, Mr = rolling torque Mrij.
// Hertz powers: ovrlp**1.5 is evaluated as ovrlp*sqrt(ovrlp) and ovrlp**0.25
// as sqrt(sqrt(ovrlp)); both agree with libm pow to ~1 ulp (the reference's
// gfortran calls pow), and cost a tenth of a double-precision pow on GB300.
__device__ __forceinline__ void force_law(const LawCfg& L, const double* P, r3 Veli, r3 Velj,
                                          r3 Rvei, r3 Rvej, double ri, double rj, r3 Norm_v,
                                          double ovrlp, dbl4& hist, r3& S, r3& M, r3& Mr) {
  r3 Vel_w = cross3(add3(scale3(Rvei, ri), scale3(Rvej, rj)), Norm_v);
  r3 Vrij = add3(sub3(Veli, Velj), Vel_w);
  double vrn = dot3(Vrij, Norm_v);
  double VelRel = hist.w;
  // comparisons run on the integer pipes (fpi::gt/lt: IEEE semantics)
  if (fpi::lt(VelRel, -1.0)) VelRel = fabs(vrn);

  r3 Vij_n = scale3(Norm_v, vrn);
  r3 Vij_t = sub3(Vrij, Vij_n);

  r3 Ovlp_t = mk3(hist.x, hist.y, hist.z);
  double normTan1 = norm3(Ovlp_t);
  Ovlp_t = sub3(Ovlp_t, scale3(Norm_v, dot3(Ovlp_t, Norm_v)));
  double normTan2 = norm3(Ovlp_t);
  if (fpi::gt(normTan2, 1.0E-10)) Ovlp_t = scale3(Ovlp_t, fpi::div_rn(normTan1, normTan2));
  else Ovlp_t = mk3(0.0, 0.0, 0.0);
  Ovlp_t = add3(scale3(Vij_t, L.dt), Ovlp_t);

  // Ftij = k_t*Ovlp_t + d_t*Vij_t with d_t = 0 (:29, :36): the second term is
  // a signed zero for finite Vij_t, and x + (+-0) == x except for the sign of a
  // zero result, which no later operation of the path can observe; it is
  // dropped (6 FP64 operations per contact).
  double fn, k_t;
  r3 Ftij;
  if (L.cf_type == SDEM_CFT_LSD) {
    double Vel_in = fpi::gt(VelRel, 0.01) ? VelRel : 0.01;
    double v04 = pow(Vel_in, 0.4);
    double k_n = -(P[SDEM_BP_KN] * v04);
    double d_n = -(P[SDEM_BP_CN] * pow(Vel_in, 0.2));
    fn = k_n * ovrlp + d_n * vrn;
    k_t = -(P[SDEM_BP_KT] * v04);
    Ftij = scale3(Ovlp_t, k_t);
  } else {
    double k_n = -P[SDEM_BP_KN];
    double d_n = -P[SDEM_BP_CN];
    double sq = fpi::sqrt_rn(ovrlp);
    double o15 = ovrlp * sq;   // ovrlp**1.5
    double o025 = fpi::sqrt_rn(sq);    // ovrlp**0.25
    fn = k_n * o15 + d_n * o025 * vrn;
    k_t = -(P[SDEM_BP_KT] * sq);
    Ftij = scale3(Ovlp_t, k_t);
  }
  r3 Fnij = scale3(Norm_v, fn);

  double ft = norm3(Ftij);
  double ft_fric = P[SDEM_BP_MUS] * fabs(fn);
  if (fpi::gt(ft, ft_fric)) {
    ft_fric = P[SDEM_BP_MUK] * fabs(fn);
    Ftij = scale3(Ftij, fpi::div_rn(ft_fric, ft));
    Ovlp_t = div3(Ftij, k_t);
  }

  r3 W_hat = sub3(Rvei, Rvej);
  double w_hat_mag = norm3(W_hat);
  if (fpi::gt(w_hat_mag, 1.0E-10)) W_hat = div3(W_hat, w_hat_mag);
  else W_hat = mk3(0.0, 0.0, 0.0);
  if (L.ct_model == SDEM_CTM_CONSTANT)
    Mr = scale3(W_hat, -(P[SDEM_BP_MUR] * fabs(fn) * P[SDEM_BP_RADEFF]));
  else
    Mr = scale3(W_hat, -(P[SDEM_BP_MUR] * fabs(fn) * P[SDEM_BP_RADEFF] * norm3(Vel_w)));

  hist = make_dbl4(Ovlp_t.x, Ovlp_t.y, Ovlp_t.z, VelRel);
  M = cross3(Norm_v, Ftij);
  S = add3(Fnij, Ftij);
}

}  // namespace sdem
