// Device spatial algebra in structured 3x3 form, FP64.
//
// Conventions (Pinocchio's): a motion is (linear, angular); a force is (force, torque);
// a placement (R, p) maps child coordinates to parent coordinates, x_parent = R x + p.
// A rigid-body inertia is kept in 10-parameter origin form (m, h = m c, I about the
// frame origin), so inertias add exactly and a 6x6 product costs 24 flops.
// Every operation here is written so that nvcc can contract it into DFMA chains: on
// GB300 the FP64 pipe, not memory, bounds these kernels.
#pragma once
#include "device_model.h"

namespace sgdyn {

struct V3 {
  double x, y, z;
};
struct M3 {  // row-major
  double a[9];
};
struct Mot {  // motion (v, w) or force (f, n)
  V3 v, w;
};
struct RBI {  // rigid-body inertia about the frame origin
  double m;
  V3 h;
  double I[6];  // xx xy xz yy yz zz
};

SG_HD V3 mk(double x, double y, double z) { return V3{x, y, z}; }
SG_HD V3 operator+(V3 a, V3 b) { return V3{a.x + b.x, a.y + b.y, a.z + b.z}; }
SG_HD V3 operator-(V3 a, V3 b) { return V3{a.x - b.x, a.y - b.y, a.z - b.z}; }
SG_HD V3 operator*(double s, V3 a) { return V3{s * a.x, s * a.y, s * a.z}; }
SG_HD V3 operator-(V3 a) { return V3{-a.x, -a.y, -a.z}; }
SG_HD double dot(V3 a, V3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
SG_HD V3 cross(V3 a, V3 b) {
  return V3{a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
}
// acc + a x b with the cross product folded into the accumulation.
SG_HD V3 add_cross(V3 acc, V3 a, V3 b) {
  return V3{fma(a.y, b.z, fma(-a.z, b.y, acc.x)), fma(a.z, b.x, fma(-a.x, b.z, acc.y)),
            fma(a.x, b.y, fma(-a.y, b.x, acc.z))};
}
SG_HD V3 axpy(double s, V3 x, V3 y) { return V3{fma(s, x.x, y.x), fma(s, x.y, y.y), fma(s, x.z, y.z)}; }

SG_HD V3 mul(const M3& R, V3 x) {
  return V3{fma(R.a[2], x.z, fma(R.a[1], x.y, R.a[0] * x.x)), fma(R.a[5], x.z, fma(R.a[4], x.y, R.a[3] * x.x)),
            fma(R.a[8], x.z, fma(R.a[7], x.y, R.a[6] * x.x))};
}
// acc + R x
SG_HD V3 mul_add(const M3& R, V3 x, V3 acc) {
  return V3{fma(R.a[2], x.z, fma(R.a[1], x.y, fma(R.a[0], x.x, acc.x))),
            fma(R.a[5], x.z, fma(R.a[4], x.y, fma(R.a[3], x.x, acc.y))),
            fma(R.a[8], x.z, fma(R.a[7], x.y, fma(R.a[6], x.x, acc.z)))};
}
SG_HD V3 mulT(const M3& R, V3 x) {
  return V3{fma(R.a[6], x.z, fma(R.a[3], x.y, R.a[0] * x.x)), fma(R.a[7], x.z, fma(R.a[4], x.y, R.a[1] * x.x)),
            fma(R.a[8], x.z, fma(R.a[5], x.y, R.a[2] * x.x))};
}
SG_HD M3 mul(const M3& A, const M3& B) {
  M3 C;
#pragma unroll
  for (int i = 0; i < 3; i++)
#pragma unroll
    for (int j = 0; j < 3; j++)
      C.a[i * 3 + j] = fma(A.a[i * 3 + 2], B.a[6 + j], fma(A.a[i * 3 + 1], B.a[3 + j], A.a[i * 3] * B.a[j]));
  return C;
}
SG_HD M3 transpose(const M3& A) {
  return M3{{A.a[0], A.a[3], A.a[6], A.a[1], A.a[4], A.a[7], A.a[2], A.a[5], A.a[8]}};
}
SG_HD M3 eye3() { return M3{{1, 0, 0, 0, 1, 0, 0, 0, 1}}; }

// Symmetric 3x3 (xx xy xz yy yz zz) times vector.
SG_HD V3 sym_mul(const double* S, V3 w) {
  return V3{fma(S[2], w.z, fma(S[1], w.y, S[0] * w.x)), fma(S[4], w.z, fma(S[3], w.y, S[1] * w.x)),
            fma(S[5], w.z, fma(S[4], w.y, S[2] * w.x))};
}
SG_HD V3 sym_mul_add(const double* S, V3 w, V3 acc) {
  return V3{fma(S[2], w.z, fma(S[1], w.y, fma(S[0], w.x, acc.x))),
            fma(S[4], w.z, fma(S[3], w.y, fma(S[1], w.x, acc.y))),
            fma(S[5], w.z, fma(S[4], w.y, fma(S[2], w.x, acc.z)))};
}

// Rotation about z with (s, c) = (sin, cos) of the angle.
SG_HD M3 rot_z(double s, double c) { return M3{{c, -s, 0, s, c, 0, 0, 0, 1}}; }
// Rotation about unit axis a by angle with (s, c) = (sin, cos): c 1 + s [a]x + (1-c) a a^T.
SG_HD M3 rodrigues(V3 a, double s, double c) {
  double t = 1.0 - c;
  double txy = t * a.x * a.y, txz = t * a.x * a.z, tyz = t * a.y * a.z;
  M3 R;
  R.a[0] = fma(t * a.x, a.x, c);
  R.a[4] = fma(t * a.y, a.y, c);
  R.a[8] = fma(t * a.z, a.z, c);
  R.a[1] = fma(-s, a.z, txy);
  R.a[3] = fma(s, a.z, txy);
  R.a[2] = fma(s, a.y, txz);
  R.a[6] = fma(-s, a.y, txz);
  R.a[5] = fma(-s, a.x, tyz);
  R.a[7] = fma(s, a.x, tyz);
  return R;
}
// Unit quaternion (x, y, z, w) -> rotation matrix.
SG_HD M3 quat_to_R(double x, double y, double z, double w) {
  double x2 = x + x, y2 = y + y, z2 = z + z;
  double xx = x * x2, yy = y * y2, zz = z * z2, xy = x * y2, xz = x * z2, yz = y * z2, wx = w * x2, wy = w * y2,
         wz = w * z2;
  return M3{{1 - (yy + zz), xy - wz, xz + wy, xy + wz, 1 - (xx + zz), yz - wx, xz - wy, yz + wx, 1 - (xx + yy)}};
}
// Rotation -> unit quaternion (w, x, y, z), Shepperd's method (largest component first).
// Case rule: the trace branch when the trace is positive, else the largest diagonal entry
// (first of equals). Written without a branch on the case: lanes of a warp hold different
// rotations, and a divergent branch would run the square root and the division once per
// case taken in the warp. The case only selects operands; the arithmetic per case is
// unchanged.
SG_HD void R_to_quat(const M3& R, double* q) {
  const double* a = R.a;
  const double t = a[0] + a[4] + a[8];
  int c = 0;  // 0: trace, 1 + i: diagonal entry i
  if (!(t > 0)) {
    int i = 0;
    if (a[4] > a[0]) i = 1;
    if (a[8] > a[i * 4]) i = 2;
    c = 1 + i;
  }
  // sqrt argument: t + 1, or R_ii - R_jj - R_kk + 1 with (i, j, k) cyclic (the diagonal
  // entries picked by selects, so that R stays in registers)
  const double di = c <= 1 ? a[0] : (c == 2 ? a[4] : a[8]);
  const double dj = c <= 1 ? a[4] : (c == 2 ? a[8] : a[0]);
  const double dk = c <= 1 ? a[8] : (c == 2 ? a[0] : a[4]);
  const double diag = di - dj - dk + 1.0;
  const double r = sqrt(c == 0 ? t + 1.0 : diag);
  const double kk = 0.5 / r;
  const double d1 = a[7] - a[5], d2 = a[2] - a[6], d3 = a[3] - a[1];
  const double s01 = a[1] + a[3], s02 = a[2] + a[6], s12 = a[5] + a[7];
  // numerators of the components not fixed to r / 2, per case (w x y z)
  const double n0 = c == 1 ? d1 : c == 2 ? d2 : d3;
  const double n1 = c == 0 ? d1 : c == 2 ? s01 : s02;
  const double n2 = c == 0 ? d2 : c == 1 ? s01 : s12;
  const double n3 = c == 0 ? d3 : c == 1 ? s02 : s12;
  const double h = 0.5 * r;
  q[0] = c == 0 ? h : n0 * kk;
  q[1] = c == 1 ? h : n1 * kk;
  q[2] = c == 2 ? h : n2 * kk;
  q[3] = c == 3 ? h : n3 * kk;
}

// Motion cross motion: a x b = (a.w x b.v + a.v x b.w, a.w x b.w); acc + a x b.
SG_HD Mot add_crossm(Mot acc, Mot a, Mot b) {
  Mot r;
  r.v = add_cross(add_cross(acc.v, a.w, b.v), a.v, b.w);
  r.w = add_cross(acc.w, a.w, b.w);
  return r;
}
// Motion cross force: v x* f = (v.w x f.f, v.w x f.n + v.v x f.f); acc + v x* f.
SG_HD Mot add_crossf(Mot acc, Mot v, Mot f) {
  Mot r;
  r.v = add_cross(acc.v, v.w, f.v);
  r.w = add_cross(add_cross(acc.w, v.w, f.w), v.v, f.v);
  return r;
}
// f = Y v with Y in origin form: (m v - h x w, I w + h x v).
SG_HD Mot rbi_mul(const RBI& Y, Mot v) {
  Mot f;
  f.v = add_cross(Y.m * v.v, v.w, Y.h);  // m v + w x h = m v - h x w
  f.w = add_cross(sym_mul(Y.I, v.w), Y.h, v.v);
  return f;
}
// acc + Y v
SG_HD Mot rbi_mul_add(const RBI& Y, Mot v, Mot acc) {
  Mot f;
  f.v = add_cross(axpy(Y.m, v.v, acc.v), v.w, Y.h);
  f.w = add_cross(sym_mul_add(Y.I, v.w, acc.w), Y.h, v.v);
  return f;
}
// Express an origin-form inertia given in a frame with pose (R, p) in the outer frame.
SG_HD RBI rbi_transport(const RBI& Y, const M3& R, V3 p) {
  // R I R^T: T = R I (I symmetric), then the upper triangle of T R^T
  const double* I = Y.I;
  double T[9];
#pragma unroll
  for (int i = 0; i < 3; i++) {
    const double r0 = R.a[i * 3], r1 = R.a[i * 3 + 1], r2 = R.a[i * 3 + 2];
    T[i * 3 + 0] = fma(r2, I[2], fma(r1, I[1], r0 * I[0]));
    T[i * 3 + 1] = fma(r2, I[4], fma(r1, I[3], r0 * I[1]));
    T[i * 3 + 2] = fma(r2, I[5], fma(r1, I[4], r0 * I[2]));
  }
  auto tr = [&](int i, int j) {
    return fma(T[i * 3 + 2], R.a[j * 3 + 2], fma(T[i * 3 + 1], R.a[j * 3 + 1], T[i * 3] * R.a[j * 3]));
  };
  V3 hr = mul(R, Y.h);
  V3 s = axpy(Y.m, p, hr);  // new first moment: R h + m p
  V3 t = s + hr;            // m p + 2 R h
  double d = fma(Y.m, dot(p, p), 2.0 * dot(hr, p));
  RBI O;
  O.m = Y.m;
  O.h = s;
  // I' = R I R^T + (m |p|^2 + 2 hr.p) 1 - p (m p + hr)^T - hr p^T
  O.I[0] = fma(-p.x, t.x, tr(0, 0) + d);
  O.I[3] = fma(-p.y, t.y, tr(1, 1) + d);
  O.I[5] = fma(-p.z, t.z, tr(2, 2) + d);
  O.I[1] = fma(-hr.x, p.y, fma(-p.x, s.y, tr(0, 1)));
  O.I[2] = fma(-hr.x, p.z, fma(-p.x, s.z, tr(0, 2)));
  O.I[4] = fma(-hr.y, p.z, fma(-p.y, s.z, tr(1, 2)));
  return O;
}

// Symmetric 6x6 spatial matrix in (linear, angular) block form [[A, B], [B^T, C]],
// A and C symmetric (xx xy xz yy yz zz), B row-major. Used for articulated inertias.
struct Sym6 {
  double A[6], B[9], C[6];
};
SG_HD Sym6 sym6_from_rbi(const RBI& Y) {
  Sym6 S;
  S.A[0] = Y.m; S.A[1] = 0; S.A[2] = 0; S.A[3] = Y.m; S.A[4] = 0; S.A[5] = Y.m;
  // B = -[h]x
  S.B[0] = 0;      S.B[1] = Y.h.z;  S.B[2] = -Y.h.y;
  S.B[3] = -Y.h.z; S.B[4] = 0;      S.B[5] = Y.h.x;
  S.B[6] = Y.h.y;  S.B[7] = -Y.h.x; S.B[8] = 0;
#pragma unroll
  for (int k = 0; k < 6; k++) S.C[k] = Y.I[k];
  return S;
}
// sym6_from_rbi(Y) + S, adding only where Y's matrix has non-zero entries
SG_HD Sym6 sym6_rbi_add(const RBI& Y, const Sym6& S) {
  Sym6 R = S;
  R.A[0] += Y.m; R.A[3] += Y.m; R.A[5] += Y.m;
  R.B[1] += Y.h.z; R.B[2] -= Y.h.y; R.B[3] -= Y.h.z;
  R.B[5] += Y.h.x; R.B[6] += Y.h.y; R.B[7] -= Y.h.x;
#pragma unroll
  for (int k = 0; k < 6; k++) R.C[k] += Y.I[k];
  return R;
}
SG_HD void sym6_acc(Sym6& P, const Sym6& S) {
#pragma unroll
  for (int k = 0; k < 6; k++) {
    P.A[k] += S.A[k];
    P.C[k] += S.C[k];
  }
#pragma unroll
  for (int k = 0; k < 9; k++) P.B[k] += S.B[k];
}
SG_HD RBI rbi_add(const RBI& a, const RBI& b) {
  RBI r;
  r.m = a.m + b.m;
  r.h = a.h + b.h;
#pragma unroll
  for (int k = 0; k < 6; k++) r.I[k] = a.I[k] + b.I[k];
  return r;
}
// acc + S x  (x a 6-vector)
SG_HD Mot sym6_mul_add(const Sym6& S, Mot x, Mot acc) {
  Mot r;
  r.v = sym_mul_add(S.A, x.v, acc.v);
  M3 B;
#pragma unroll
  for (int k = 0; k < 9; k++) B.a[k] = S.B[k];
  r.v = mul_add(B, x.w, r.v);
  r.w = sym_mul_add(S.C, x.w, mulT(B, x.v) + acc.w);
  return r;
}
SG_HD Mot sym6_mul(const Sym6& S, Mot x) {
  Mot z{{0, 0, 0}, {0, 0, 0}};
  return sym6_mul_add(S, x, z);
}
SG_HD double dot6(Mot a, Mot b) {
  return fma(a.w.z, b.w.z, fma(a.w.y, b.w.y, fma(a.w.x, b.w.x, fma(a.v.z, b.v.z, fma(a.v.y, b.v.y, a.v.x * b.v.x)))));
}
SG_HD Mot scale6(double s, Mot a) { return Mot{s * a.v, s * a.w}; }
SG_HD Mot axpy6(double s, Mot x, Mot y) { return Mot{axpy(s, x.v, y.v), axpy(s, x.w, y.w)}; }
SG_HD Mot add6(Mot a, Mot b) { return Mot{a.v + b.v, a.w + b.w}; }

}  // namespace sgdyn
