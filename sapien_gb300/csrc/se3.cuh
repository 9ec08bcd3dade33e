// SE(3) exponential, logarithm and the Jacobian of the logarithm, FP64 device code.
//
// log3 goes through the rotation's unit quaternion (Shepperd extraction, then
// theta = 2 atan2(|v|, w) with w >= 0), which stays well conditioned up to theta = pi.
// log6(M) = (alpha p - 1/2 w x p + beta (w.p) w, w) with beta = g(theta),
// alpha = 1 - theta^2 g(theta), g(t) = (1 - (t/2) cot(t/2)) / t^2.
// Jlog6(M) is the derivative for a right perturbation, log6(M exp6(d)) ~ log6(M) + J d,
// i.e. the inverse of the SE(3) right Jacobian J_r(xi) = J_l(-xi) in Barfoot's block
// form [[J, Q], [0, J]] (T. Barfoot, "State Estimation for Robotics", 2017, sec. 7.1.5);
// it depends on M only through xi = log6(M), and log6(M^-1) = -log6(M).
// Coefficient functions switch to their Taylor series below fixed thresholds so no
// branch loses precision to cancellation.
#pragma once
#include "spatial.cuh"

namespace sgdyn {

// sum_k c[k] x^k by Horner's rule; with a constant table and full unrolling this is K - 1
// FMAs, no division.
template <int K>
SG_HD double se3_horner(const double (&c)[K], double x) {
  double r = c[K - 1];
#pragma unroll
  for (int k = K - 2; k >= 0; k--) r = fma(r, x, c[k]);
  return r;
}

// Series coefficients below are the exact rationals rounded to the nearest double.
SG_HD double se3_f_1mc(double t) {  // (1 - cos t) / t^2 = sum (-1)^k t^2k / (2k+2)!
  if (t < 0.3) {
    const double c[10] = {0.5, -0.041666666666666664, 0.001388888888888889, -2.48015873015873e-05,
                          2.755731922398589e-07, -2.08767569878681e-09, 1.1470745597729725e-11,
                          -4.779477332387385e-14, 1.5619206968586225e-16, -4.110317623312165e-19};
    return se3_horner(c, t * t);
  }
  return (1 - cos(t)) / (t * t);
}
SG_HD double se3_f_sinc(double t) {  // sin t / t = sum (-1)^k t^2k / (2k+1)!
  if (t < 0.3) {
    const double c[10] = {1.0, -0.16666666666666666, 0.008333333333333333, -0.0001984126984126984,
                          2.7557319223985893e-06, -2.505210838544172e-08, 1.6059043836821613e-10,
                          -7.647163731819816e-13, 2.8114572543455206e-15, -8.22063524662433e-18};
    return se3_horner(c, t * t);
  }
  return sin(t) / t;
}
SG_HD double se3_f_tms(double t) {  // (t - sin t) / t^3 = sum (-1)^k t^2k / (2k+3)!
  if (t < 0.3) {
    const double c[10] = {0.16666666666666666, -0.008333333333333333, 0.0001984126984126984,
                          -2.7557319223985893e-06, 2.505210838544172e-08, -1.6059043836821613e-10,
                          7.647163731819816e-13, -2.8114572543455206e-15, 8.22063524662433e-18,
                          -1.9572941063391263e-20};
    return se3_horner(c, t * t);
  }
  return (t - sin(t)) / (t * t * t);
}
// (t^2 + 2 cos t - 2) / (2 t^4) = sum (-1)^k t^2k / (2k+4)!
SG_HD double se3_f_c4(double t) {
  if (t < 0.6) {
    const double c[12] = {0.041666666666666664, -0.001388888888888889, 2.48015873015873e-05,
                          -2.755731922398589e-07, 2.08767569878681e-09, -1.1470745597729725e-11,
                          4.779477332387385e-14, -1.5619206968586225e-16, 4.110317623312165e-19,
                          -8.896791392450574e-22, 1.6117375710961184e-24, -2.4795962632247976e-27};
    return se3_horner(c, t * t);
  }
  return (t * t + 2 * cos(t) - 2) / (2 * t * t * t * t);
}
// (2t - 3 sin t + t cos t) / (2 t^5) = sum_{n>=2} (-1)^n (n-1) t^(2n-4) / (2n+1)!
SG_HD double se3_f_c5(double t) {
  if (t < 0.9) {
    const double c[14] = {0.008333333333333333, -0.0003968253968253968, 8.267195767195768e-06,
                          -1.0020843354176688e-07, 8.029521918410807e-10, -4.58829823909189e-12,
                          1.9680200780418645e-14, -6.576508197299464e-17, 1.7615646957052136e-19,
                          -3.868170170630684e-22, 7.091645312822921e-25, -1.1020427836554655e-27,
                          1.4702951752382032e-30, -1.7025750581749252e-33};
    return se3_horner(c, t * t);
  }
  return (2 * t - 3 * sin(t) + t * cos(t)) / (2 * t * t * t * t * t);
}
SG_HD double se3_f_g(double t) {  // (1 - (t/2) cot(t/2)) / t^2
  if (t < 0.3) {
    const double c[6] = {1.0 / 12, 1.0 / 720, 1.0 / 30240, 1.0 / 1209600, 1.0 / 47900160, 691.0 / 1307674368000.0};
    return se3_horner(c, t * t);
  }
  double h = 0.5 * t;
  return (1 - h * cos(h) / sin(h)) / (t * t);
}

SG_HD M3 skew3(V3 w) { return M3{{0, -w.z, w.y, w.z, 0, -w.x, -w.y, w.x, 0}}; }
SG_HD M3 add3(const M3& A, const M3& B) {
  M3 C;
#pragma unroll
  for (int k = 0; k < 9; k++) C.a[k] = A.a[k] + B.a[k];
  return C;
}

// Rotation vector of R (theta in [0, pi]).
SG_HD V3 log3(const M3& R, double* theta) {
  double q[4];
  R_to_quat(R, q);
  if (q[0] < 0) {
    q[0] = -q[0];
    q[1] = -q[1];
    q[2] = -q[2];
    q[3] = -q[3];
  }
  double n = sqrt(q[1] * q[1] + q[2] * q[2] + q[3] * q[3]);
  if (n == 0) {
    *theta = 0;
    return mk(0, 0, 0);
  }
  double th = 2 * atan2(n, q[0]);
  *theta = th;
  double k = th / n;
  return mk(k * q[1], k * q[2], k * q[3]);
}

// log6 of (R, p): linear part, angular part.
SG_HD Mot log6(const M3& R, V3 p) {
  double t;
  V3 w = log3(R, &t);
  double beta = se3_f_g(t);
  double alpha = 1 - t * t * beta;
  V3 wxp = cross(w, p);
  double wp = dot(w, p);
  Mot out;
  out.v = mk(alpha * p.x - 0.5 * wxp.x + beta * wp * w.x, alpha * p.y - 0.5 * wxp.y + beta * wp * w.y,
             alpha * p.z - 0.5 * wxp.z + beta * wp * w.z);
  out.w = w;
  return out;
}

// exp6 of (v, w) -> (R, p): R = 1 + sinc(t) K + f_1mc(t) K^2, p = (1 + f_1mc(t) K + f_tms(t) K^2) v
// with K = [w]x, t = |w|.
SG_HD void exp6(Mot nu, M3& R, V3& p) {
  V3 w = nu.w;
  double t = sqrt(dot(w, w));
  M3 K = skew3(w), K2 = mul(K, K);
  double a = se3_f_sinc(t), b = se3_f_1mc(t), c = se3_f_tms(t);
  M3 V = eye3();
  R = eye3();
#pragma unroll
  for (int k = 0; k < 9; k++) {
    V.a[k] += b * K.a[k] + c * K2.a[k];
    R.a[k] += a * K.a[k] + b * K2.a[k];
  }
  p = mul(V, nu.v);
}

// Free-flyer configuration q = (x y z qx qy qz qw) advanced by the body twist v (linear,
// angular): (R, p) <- (R, p) exp6(v) (Pinocchio's integrate), the new quaternion taken on
// the same hemisphere as the old one and renormalised. In place.
SG_HD void free_flyer_integrate(double* q, const double* v) {
  const M3 R0 = quat_to_R(q[3], q[4], q[5], q[6]);
  M3 dR;
  V3 dp;
  exp6(Mot{mk(v[0], v[1], v[2]), mk(v[3], v[4], v[5])}, dR, dp);
  const M3 R1 = mul(R0, dR);
  const V3 p1 = mul_add(R0, dp, mk(q[0], q[1], q[2]));
  double qw[4];
  R_to_quat(R1, qw);  // w x y z
  const double dq = qw[1] * q[3] + qw[2] * q[4] + qw[3] * q[5] + qw[0] * q[6];
  const double s = (dq < 0 ? -1.0 : 1.0) / sqrt(qw[0] * qw[0] + qw[1] * qw[1] + qw[2] * qw[2] + qw[3] * qw[3]);
  q[0] = p1.x;
  q[1] = p1.y;
  q[2] = p1.z;
  q[3] = s * qw[1];
  q[4] = s * qw[2];
  q[5] = s * qw[3];
  q[6] = s * qw[0];
}

// Semi-implicit Euler on one environment's rows: qd += dt qdd, then q advanced by dt qd
// (angles and slides add; a free flyer moves on SE(3) by its body twist dt qd).
template <class Tab>
SG_HD void integrate_env_t(const Tab& T, double* q, double* qd, const double* qdd, double dt) {
#pragma unroll
  for (int i = 1; i < T.nj(); i++) {
    const DJoint& J = T.joint(i);
    if (J.kind == JK_FREEFLYER) {
      double v[6];
#pragma unroll
      for (int k = 0; k < 6; k++) {
        const double w = fma(dt, qdd[J.vcol + k], qd[J.vcol + k]);
        qd[J.vcol + k] = w;
        v[k] = dt * w;
      }
      free_flyer_integrate(q + J.qcol, v);
    } else {
      const double w = fma(dt, qdd[J.vcol], qd[J.vcol]);
      qd[J.vcol] = w;
      q[J.qcol] = fma(dt, w, q[J.qcol]);
    }
  }
}

// Jlog6 of the transform whose log6 is xi = (rho, phi), as its blocks: Jlog6 =
// [[Jinv, -TR], [0, Jinv]] in (linear, angular) ordering, with Jinv = 1 + 1/2 [phi]x +
// g(t) [phi]x^2 and TR = Jinv Q Jinv, Q = Q_l(-rho, -phi). The skew products in Barfoot's
// Q reduce to outer products (d = phi.rho, [a]x[b]x = b a^T - (a.b) 1, and
// [phi]x [rho]x [phi]x = -d [phi]x):
//   Q = -1/2 [rho]x + a (rho phi^T + phi rho^T - 2d 1 + d [phi]x)
//       + b (phi (phi x rho)^T - (phi x rho) phi^T - d [phi]x) - 2 c d (phi phi^T - t^2 1)
// with a = f_tms(t), b = f_c4(t), c = f_c5(t).
SG_HD void jlog6_blocks(const Mot& xi, M3& Jinv, M3& TR) {
  const V3 rho = xi.v, phi = xi.w;
  const double t2 = dot(phi, phi), t = sqrt(t2), d = dot(phi, rho);
  const double g = se3_f_g(t), a = se3_f_tms(t), b = se3_f_c4(t), c = se3_f_c5(t);
  const double f[3] = {phi.x, phi.y, phi.z}, r[3] = {rho.x, rho.y, rho.z};
  const V3 fxr = cross(phi, rho);
  const double u[3] = {fxr.x, fxr.y, fxr.z};  // phi x rho
  const M3 Kf = skew3(phi), Kr = skew3(rho);
  M3 Q;
#pragma unroll
  for (int i = 0; i < 3; i++)
#pragma unroll
    for (int k = 0; k < 3; k++) {
      const double id = i == k ? 1.0 : 0.0;
      const double ppT = f[i] * f[k] - t2 * id;  // [phi]x^2
      Jinv.a[i * 3 + k] = id + 0.5 * Kf.a[i * 3 + k] + g * ppT;
      Q.a[i * 3 + k] = -0.5 * Kr.a[i * 3 + k] + a * (r[i] * f[k] + f[i] * r[k] - 2 * d * id + d * Kf.a[i * 3 + k]) +
                       b * (f[i] * u[k] - u[i] * f[k] - d * Kf.a[i * 3 + k]) - 2 * c * d * ppT;
    }
  TR = mul(mul(Jinv, Q), Jinv);
}

// Adjoint of the free-flyer integrate q' = q exp6(delta) (right perturbations, body
// twists): given the adjoint g of q', returns the adjoint of q, Ad(exp6(-delta))^T g, and
// adds dt J_r(delta)^T g to the adjoint of the velocity that made delta = dt v. Here
// J_r(delta) = [[J, Q], [0, J]] is the right Jacobian of SE(3), q exp6(delta + eta) ~
// q exp6(delta) exp6(J_r eta), with J = 1 - f_1mc(t) [phi]x + f_tms(t) [phi]x^2 and Q the
// block of jlog6_blocks (whose Jinv, -TR are the blocks of J_r^-1), delta = (rho, phi).
// Ad(R, p)^T (a, b) = (R^T a, R^T (b - p x a)).
SG_HD Mot free_flyer_integrate_adjoint(const Mot& delta, const Mot& g, double dt, Mot& vbar) {
  const V3 rho = delta.v, phi = delta.w;
  const double t2 = dot(phi, phi), t = sqrt(t2), d = dot(phi, rho);
  const double b1 = se3_f_1mc(t), c1 = se3_f_tms(t);
  const double a = se3_f_tms(t), b = se3_f_c4(t), c = se3_f_c5(t);
  const double f[3] = {phi.x, phi.y, phi.z}, r[3] = {rho.x, rho.y, rho.z};
  const V3 fxr = cross(phi, rho);
  const double u[3] = {fxr.x, fxr.y, fxr.z};
  const M3 Kf = skew3(phi), Kr = skew3(rho);
  M3 J, Q;
#pragma unroll
  for (int i = 0; i < 3; i++)
#pragma unroll
    for (int k = 0; k < 3; k++) {
      const double id = i == k ? 1.0 : 0.0;
      const double ppT = f[i] * f[k] - t2 * id;
      J.a[i * 3 + k] = id - b1 * Kf.a[i * 3 + k] + c1 * ppT;
      Q.a[i * 3 + k] = -0.5 * Kr.a[i * 3 + k] + a * (r[i] * f[k] + f[i] * r[k] - 2 * d * id + d * Kf.a[i * 3 + k]) +
                       b * (f[i] * u[k] - u[i] * f[k] - d * Kf.a[i * 3 + k]) - 2 * c * d * ppT;
    }
  // J_r^T g = (J^T g_lin, Q^T g_lin + J^T g_ang)
  vbar.v = vbar.v + dt * mulT(J, g.v);
  vbar.w = vbar.w + dt * (mulT(Q, g.v) + mulT(J, g.w));
  M3 Re;
  V3 pe;
  exp6(Mot{-delta.v, -delta.w}, Re, pe);
  return Mot{mulT(Re, g.v), mulT(Re, g.w - cross(pe, g.v))};
}

}  // namespace sgdyn
