// CPU FP64 oracle for the articulated-body dynamics path (TEST INFRASTRUCTURE ONLY).
//
// Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg may load this
// library, and only as the checker / reported CPU baseline. The product path never
// calls it.
//
// What it restates. The reference computes this path through sapien::PinocchioModel
// (pinocchio/pinocchio_model.cpp), a thin wrapper whose arithmetic lives in the
// third-party Pinocchio v2.6.18 library (pinocchio/cmake/pinocchio.cmake:46-53),
// which is not present in the reference tree and cannot be built here (it needs
// Eigen 3.4, Boost 1.81, urdfdom fetched from the network). This file therefore
// restates, in its own code:
//   * the wrapper semantics of pinocchio/pinocchio_model.cpp: posS2P / posP2S
//     (:49-97), the S<->P joint permutation (:99-128), link frames (:130-140),
//     getLinkPose composition (:150-161), getLinkJacobian world/local (:167-186),
//     computeSingleLinkLocalJacobian (:188-199), CRBA symmetrisation (:201-206),
//     Coriolis (:208-212), RNEA (:214-219), ABA (:221-226) and the CLIK loop with
//     best-iterate tracking, eps / max-iteration exits, Jlog6 and damped LDLT
//     step (:228-300);
//   * Pinocchio's published conventions: motion vectors ordered (linear, angular),
//     SE3 placements mapping child to parent, local-frame RNEA and ABA
//     (Featherstone, "Rigid Body Dynamics Algorithms", 2008, ch. 5 and 7), WORLD
//     Jacobian columns oMi.act(S), CRBA, log6/Jlog6 on SE(3) and the free-flyer /
//     unbounded-revolute integrators.
// Everything is written with dense 6x6 Plucker matrices on purpose: the GPU kernels
// use structured 3x3 algebra, so the two implementations share no arithmetic
// shortcuts.
//
// Parity status: parity unpinned. The reference's only test touching this path
// (unittest/test_physx/test_articulation.py:75-97) compares against PhysX at run
// time and holds no golden numbers; this oracle is pinned instead by closed forms
// and identities checked in tests/test_oracle.py.
#include <algorithm>
#include <array>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <thread>
#include <vector>

// ---- counting scalar ---------------------------------------------------------------
// Cnt carries a double and counts the floating-point operations the templated algorithms
// below perform on it, per thread. Operations whose result needs no arithmetic are not
// counted: a product with an exact 0, 1 or -1 operand, a sum or difference with an exact 0
// operand, a division by +-1, a negation. The dense 6x6 Plucker matrices of this oracle
// hold such structural zeros and ones (the zero block of a motion transform, unit motion
// subspaces, identity placements), so the counts are those of the same recursions with
// the structure exploited, i.e. the algorithm's own work rather than this restatement's
// dense storage. sqrt, divisions and transcendental calls are counted apart.
namespace orc_count {
struct Counts {
  long long add = 0, mul = 0, div = 0, sqrt = 0, trig = 0;
};
inline thread_local Counts g_counts;
struct Cnt {
  double v = 0;
  Cnt() = default;
  Cnt(double x) : v(x) {}
  explicit operator double() const { return v; }
  Cnt& operator+=(Cnt b);
  Cnt& operator-=(Cnt b);
  Cnt& operator*=(Cnt b);
  Cnt& operator/=(Cnt b);
};
inline bool unit(double x) { return x == 1.0 || x == -1.0; }
inline Cnt operator+(Cnt a, Cnt b) {
  if (a.v != 0 && b.v != 0) g_counts.add++;
  return Cnt(a.v + b.v);
}
inline Cnt operator-(Cnt a, Cnt b) {
  if (a.v != 0 && b.v != 0) g_counts.add++;
  return Cnt(a.v - b.v);
}
inline Cnt operator*(Cnt a, Cnt b) {
  if (a.v != 0 && b.v != 0 && !unit(a.v) && !unit(b.v)) g_counts.mul++;
  return Cnt(a.v * b.v);
}
inline Cnt operator/(Cnt a, Cnt b) {
  if (a.v != 0 && !unit(b.v)) g_counts.div++;
  return Cnt(a.v / b.v);
}
inline Cnt operator-(Cnt a) { return Cnt(-a.v); }
inline Cnt& Cnt::operator+=(Cnt b) { return *this = *this + b; }
inline Cnt& Cnt::operator-=(Cnt b) { return *this = *this - b; }
inline Cnt& Cnt::operator*=(Cnt b) { return *this = *this * b; }
inline Cnt& Cnt::operator/=(Cnt b) { return *this = *this / b; }
inline bool operator<(Cnt a, Cnt b) { return a.v < b.v; }
inline bool operator>(Cnt a, Cnt b) { return a.v > b.v; }
inline bool operator<=(Cnt a, Cnt b) { return a.v <= b.v; }
inline bool operator>=(Cnt a, Cnt b) { return a.v >= b.v; }
inline bool operator==(Cnt a, Cnt b) { return a.v == b.v; }
inline bool operator!=(Cnt a, Cnt b) { return a.v != b.v; }
}  // namespace orc_count

// math functions on the counting scalar, found by the std:: calls in the templates
namespace std {
inline orc_count::Cnt sqrt(orc_count::Cnt x) {
  orc_count::g_counts.sqrt++;
  return orc_count::Cnt(std::sqrt(x.v));
}
inline orc_count::Cnt sin(orc_count::Cnt x) {
  orc_count::g_counts.trig++;
  return orc_count::Cnt(std::sin(x.v));
}
inline orc_count::Cnt cos(orc_count::Cnt x) {
  orc_count::g_counts.trig++;
  return orc_count::Cnt(std::cos(x.v));
}
inline orc_count::Cnt atan2(orc_count::Cnt y, orc_count::Cnt x) {
  orc_count::g_counts.trig++;
  return orc_count::Cnt(std::atan2(y.v, x.v));
}
inline orc_count::Cnt fabs(orc_count::Cnt x) { return orc_count::Cnt(std::fabs(x.v)); }
}  // namespace std

namespace {

constexpr int kMaxJ = 96;   // joints incl. universe
constexpr int kMaxV = 128;  // velocity dimension

enum JType { JT_UNIVERSE = 0, JT_REVOLUTE = 1, JT_PRISMATIC = 2, JT_CONTINUOUS = 3, JT_FREEFLYER = 4 };

template <class S> using V3 = std::array<S, 3>;
template <class S> using M3 = std::array<S, 9>;  // row-major
template <class S> using V6 = std::array<S, 6>;
template <class S> using M6 = std::array<S, 36>;  // row-major

template <class S> struct SE3 {
  M3<S> R;
  V3<S> p;
};

template <class S> M3<S> eye3() { return {1, 0, 0, 0, 1, 0, 0, 0, 1}; }
template <class S> M3<S> mul3(const M3<S>& A, const M3<S>& B) {
  M3<S> C{};
  for (int i = 0; i < 3; i++)
    for (int j = 0; j < 3; j++) {
      S s = 0;
      for (int k = 0; k < 3; k++) s += A[i * 3 + k] * B[k * 3 + j];
      C[i * 3 + j] = s;
    }
  return C;
}
template <class S> V3<S> mv3(const M3<S>& A, const V3<S>& x) {
  V3<S> y{};
  for (int i = 0; i < 3; i++) y[i] = A[i * 3] * x[0] + A[i * 3 + 1] * x[1] + A[i * 3 + 2] * x[2];
  return y;
}
template <class S> M3<S> tr3(const M3<S>& A) {
  M3<S> B{};
  for (int i = 0; i < 3; i++)
    for (int j = 0; j < 3; j++) B[i * 3 + j] = A[j * 3 + i];
  return B;
}
template <class S> M3<S> skew(const V3<S>& v) { return {0, -v[2], v[1], v[2], 0, -v[0], -v[1], v[0], 0}; }
template <class S> V3<S> cross(const V3<S>& a, const V3<S>& b) {
  return {a[1] * b[2] - a[2] * b[1], a[2] * b[0] - a[0] * b[2], a[0] * b[1] - a[1] * b[0]};
}
template <class S> S dot3(const V3<S>& a, const V3<S>& b) { return a[0] * b[0] + a[1] * b[1] + a[2] * b[2]; }
template <class S> M3<S> add3(const M3<S>& A, const M3<S>& B) {
  M3<S> C;
  for (int i = 0; i < 9; i++) C[i] = A[i] + B[i];
  return C;
}
template <class S> M3<S> scale3(const M3<S>& A, S s) {
  M3<S> C;
  for (int i = 0; i < 9; i++) C[i] = A[i] * s;
  return C;
}

template <class S> SE3<S> se3mul(const SE3<S>& a, const SE3<S>& b) {
  SE3<S> c;
  c.R = mul3(a.R, b.R);
  V3<S> t = mv3(a.R, b.p);
  for (int i = 0; i < 3; i++) c.p[i] = t[i] + a.p[i];
  return c;
}
template <class S> SE3<S> se3inv(const SE3<S>& a) {
  SE3<S> c;
  c.R = tr3(a.R);
  V3<S> t = mv3(c.R, a.p);
  for (int i = 0; i < 3; i++) c.p[i] = -t[i];
  return c;
}
template <class S> SE3<S> se3id() { return {eye3<S>(), {0, 0, 0}}; }

// 6x6 helpers (row-major)
template <class S> M6<S> mul6(const M6<S>& A, const M6<S>& B) {
  M6<S> C{};
  for (int i = 0; i < 6; i++)
    for (int j = 0; j < 6; j++) {
      S s = 0;
      for (int k = 0; k < 6; k++) s += A[i * 6 + k] * B[k * 6 + j];
      C[i * 6 + j] = s;
    }
  return C;
}
template <class S> V6<S> mv6(const M6<S>& A, const V6<S>& x) {
  V6<S> y{};
  for (int i = 0; i < 6; i++) {
    S s = 0;
    for (int k = 0; k < 6; k++) s += A[i * 6 + k] * x[k];
    y[i] = s;
  }
  return y;
}
template <class S> M6<S> tr6(const M6<S>& A) {
  M6<S> B{};
  for (int i = 0; i < 6; i++)
    for (int j = 0; j < 6; j++) B[i * 6 + j] = A[j * 6 + i];
  return B;
}
template <class S> void put3(M6<S>& A, int r, int c, const M3<S>& B) {
  for (int i = 0; i < 3; i++)
    for (int j = 0; j < 3; j++) A[(r + i) * 6 + c + j] = B[i * 3 + j];
}
// Motion action of M: [R, [p]x R; 0, R]
template <class S> M6<S> act6(const SE3<S>& M) {
  M6<S> X{};
  put3(X, 0, 0, M.R);
  put3(X, 3, 3, M.R);
  put3(X, 0, 3, mul3(skew(M.p), M.R));
  return X;
}
template <class S> M6<S> actinv6(const SE3<S>& M) { return act6(se3inv(M)); }
// v x (motion cross): [w^, v^; 0, w^]
template <class S> M6<S> crm(const V6<S>& v) {
  M6<S> X{};
  V3<S> lin{v[0], v[1], v[2]}, ang{v[3], v[4], v[5]};
  put3(X, 0, 0, skew(ang));
  put3(X, 3, 3, skew(ang));
  put3(X, 0, 3, skew(lin));
  return X;
}
// v x* (force cross) = -crm(v)^T
template <class S> M6<S> crf(const V6<S>& v) {
  M6<S> X = tr6(crm(v));
  for (auto& x : X) x = -x;
  return X;
}
template <class S> V6<S> addv6(const V6<S>& a, const V6<S>& b) {
  V6<S> c;
  for (int i = 0; i < 6; i++) c[i] = a[i] + b[i];
  return c;
}

template <class S> M3<S> quat_to_R(S x, S y, S z, S w) {
  return {1 - 2 * (y * y + z * z), 2 * (x * y - w * z),     2 * (x * z + w * y),
          2 * (x * y + w * z),     1 - 2 * (x * x + z * z), 2 * (y * z - w * x),
          2 * (x * z - w * y),     2 * (y * z + w * x),     1 - 2 * (x * x + y * y)};
}
// Rotation -> unit quaternion (w, x, y, z) by Shepperd's method (the largest of
// w, x, y, z is extracted first; w >= 0 when trace > 0).
template <class S> std::array<S, 4> R_to_quat(const M3<S>& R) {
  std::array<S, 4> q;  // w x y z
  S t = R[0] + R[4] + R[8];
  if (t > 0) {
    S r = std::sqrt(t + 1);
    q[0] = S(0.5) * r;
    r = S(0.5) / r;
    q[1] = (R[7] - R[5]) * r;
    q[2] = (R[2] - R[6]) * r;
    q[3] = (R[3] - R[1]) * r;
  } else {
    int i = 0;
    if (R[4] > R[0]) i = 1;
    if (R[8] > R[i * 4]) i = 2;
    int j = (i + 1) % 3, k = (j + 1) % 3;
    S r = std::sqrt(R[i * 4] - R[j * 4] - R[k * 4] + 1);
    q[1 + i] = S(0.5) * r;
    r = S(0.5) / r;
    q[0] = (R[k * 3 + j] - R[j * 3 + k]) * r;
    q[1 + j] = (R[j * 3 + i] + R[i * 3 + j]) * r;
    q[1 + k] = (R[k * 3 + i] + R[i * 3 + k]) * r;
  }
  return q;
}

// Rodrigues rotation about unit axis a given (sin, cos).
template <class S> M3<S> rodrigues(const V3<S>& a, S s, S c) {
  M3<S> K = skew(a);
  M3<S> K2 = mul3(K, K);
  M3<S> R = eye3<S>();
  for (int i = 0; i < 9; i++) R[i] += s * K[i] + (1 - c) * K2[i];
  return R;
}

// ---- SE(3) / SO(3) exponential, logarithm and Jacobians -------------------
// Coefficient functions with series branches (terms in theta^2) near zero.
template <class S> S f_1mc(S t) {  // (1 - cos t) / t^2
  if (t < S(0.3)) {
    S t2 = t * t, r = 0, term = S(0.5);
    for (int k = 0; k < 10; k++) { r += term; term *= -t2 / S((2 * k + 3) * (2 * k + 4)); }
    return r;
  }
  return (1 - std::cos(t)) / (t * t);
}
template <class S> S f_tms(S t) {  // (t - sin t) / t^3
  if (t < S(0.3)) {
    S t2 = t * t, r = 0, term = S(1) / 6;
    for (int k = 0; k < 10; k++) { r += term; term *= -t2 / S((2 * k + 4) * (2 * k + 5)); }
    return r;
  }
  return (t - std::sin(t)) / (t * t * t);
}
template <class S> S f_c4(S t) {  // (t^2 + 2 cos t - 2) / (2 t^4)
  if (t < S(0.6)) {
    S t2 = t * t, r = 0, term = S(1) / 24;
    for (int k = 0; k < 12; k++) { r += term; term *= -t2 / S((2 * k + 5) * (2 * k + 6)); }
    return r;
  }
  return (t * t + 2 * std::cos(t) - 2) / (2 * t * t * t * t);
}
template <class S> S f_c5(S t) {  // (2t - 3 sin t + t cos t) / (2 t^5)
  if (t < S(0.9)) {
    // sum_{n>=2} (-1)^n (n-1) t^(2n-4) / (2n+1)!
    S t2 = t * t, r = 0, fact = 120, pw = 1;
    for (int n = 2; n < 16; n++) {
      r += ((n % 2) ? -1 : 1) * S(n - 1) * pw / fact;
      pw *= t2;
      fact *= S((2 * n + 2) * (2 * n + 3));
    }
    return r;
  }
  return (2 * t - 3 * std::sin(t) + t * std::cos(t)) / (2 * t * t * t * t * t);
}
// g(t) = (1 - (t/2) cot(t/2)) / t^2 = sum_{k>=1} |B_2k| t^(2k-2) / (2k)!
template <class S> S f_g(S t) {
  if (t < S(0.3)) {
    const double c[] = {1.0 / 12, 1.0 / 720, 1.0 / 30240, 1.0 / 1209600, 1.0 / 47900160, 691.0 / 1307674368000.0};
    S t2 = t * t, r = 0, pw = 1;
    for (double ci : c) { r += S(ci) * pw; pw *= t2; }
    return r;
  }
  S h = t / 2;
  return (1 - h * std::cos(h) / std::sin(h)) / (t * t);
}

template <class S> M3<S> exp3(const V3<S>& w) {
  S t = std::sqrt(dot3(w, w));
  M3<S> K = skew(w), K2 = mul3(K, K);
  S a = (t < S(0.3)) ? [&] {  // sin t / t
    S t2 = t * t, r = 0, term = 1;
    for (int k = 0; k < 10; k++) { r += term; term *= -t2 / S((2 * k + 2) * (2 * k + 3)); }
    return r;
  }() : std::sin(t) / t;
  S b = f_1mc(t);
  M3<S> R = eye3<S>();
  for (int i = 0; i < 9; i++) R[i] += a * K[i] + b * K2[i];
  return R;
}
// Rotation vector of R via its quaternion: theta = 2 atan2(|v|, w) with w >= 0.
template <class S> V3<S> log3(const M3<S>& R, S* theta_out = nullptr) {
  auto q = R_to_quat(R);
  if (q[0] < 0) for (auto& x : q) x = -x;
  S n = std::sqrt(q[1] * q[1] + q[2] * q[2] + q[3] * q[3]);
  if (n == 0) {
    if (theta_out) *theta_out = 0;
    return {0, 0, 0};
  }
  S th = 2 * std::atan2(n, q[0]);
  if (theta_out) *theta_out = th;
  S k = th / n;
  return {k * q[1], k * q[2], k * q[3]};
}
// SE(3) exponential of (v, w).
template <class S> SE3<S> exp6(const V6<S>& nu) {
  V3<S> v{nu[0], nu[1], nu[2]}, w{nu[3], nu[4], nu[5]};
  S t = std::sqrt(dot3(w, w));
  M3<S> K = skew(w), K2 = mul3(K, K);
  M3<S> V = eye3<S>();
  S b = f_1mc(t), c = f_tms(t);
  for (int i = 0; i < 9; i++) V[i] += b * K[i] + c * K2[i];
  SE3<S> M;
  M.R = exp3(w);
  M.p = mv3(V, v);
  return M;
}
// SE(3) logarithm (linear, angular).
template <class S> V6<S> log6(const SE3<S>& M) {
  S t;
  V3<S> w = log3(M.R, &t);
  S beta = f_g(t);
  S alpha = 1 - t * t * beta;
  V3<S> wxp = cross(w, M.p);
  S wp = dot3(w, M.p);
  V6<S> out;
  for (int i = 0; i < 3; i++) out[i] = alpha * M.p[i] - S(0.5) * wxp[i] + beta * wp * w[i];
  for (int i = 0; i < 3; i++) out[3 + i] = w[i];
  return out;
}
// Right Jacobian inverse of SO(3): I + 1/2 [w] + g(t) [w]^2.
template <class S> M3<S> jlog3(const V3<S>& w) {
  S t = std::sqrt(dot3(w, w));
  M3<S> K = skew(w), K2 = mul3(K, K);
  S g = f_g(t);
  M3<S> J = eye3<S>();
  for (int i = 0; i < 9; i++) J[i] += S(0.5) * K[i] + g * K2[i];
  return J;
}
// Barfoot's Q_l(rho, phi) block of the SE(3) left Jacobian.
template <class S> M3<S> q_left(const V3<S>& rho, const V3<S>& phi) {
  S t = std::sqrt(dot3(phi, phi));
  M3<S> P = skew(phi), Rh = skew(rho);
  M3<S> PR = mul3(P, Rh), RP = mul3(Rh, P), PRP = mul3(PR, P);
  M3<S> PPR = mul3(P, PR), RPP = mul3(RP, P), PRPP = mul3(PRP, P), PPRP = mul3(P, PRP);
  S a = f_tms(t), b = f_c4(t), c = f_c5(t);
  M3<S> Q;
  for (int i = 0; i < 9; i++)
    Q[i] = S(0.5) * Rh[i] + a * (PR[i] + RP[i] + PRP[i]) + b * (PPR[i] + RPP[i] - 3 * PRP[i]) +
           c * (PRPP[i] + PPRP[i]);
  return Q;
}
// Jlog6(M): derivative of log6 for a right (local) perturbation,
// log6(M exp6(d)) ~ log6(M) + Jlog6(M) d. Equals J_r(xi)^-1 with J_r(xi) = J_l(-xi).
template <class S> M6<S> jlog6(const SE3<S>& M) {
  V6<S> xi = log6(M);
  V3<S> rho{xi[0], xi[1], xi[2]}, phi{xi[3], xi[4], xi[5]};
  M3<S> Jinv = jlog3(phi);
  M3<S> Qr = q_left(V3<S>{-rho[0], -rho[1], -rho[2]}, V3<S>{-phi[0], -phi[1], -phi[2]});
  M3<S> TR = mul3(mul3(Jinv, Qr), Jinv);
  M6<S> J{};
  put3(J, 0, 0, Jinv);
  put3(J, 3, 3, Jinv);
  for (int i = 0; i < 9; i++) TR[i] = -TR[i];
  put3(J, 0, 3, TR);
  return J;
}

// Generic dense solvers for small SPD / general systems.
template <class S> bool chol_solve(int n, std::vector<S> A, S* b) {  // A row-major n x n
  for (int j = 0; j < n; j++) {
    S d = A[j * n + j];
    for (int k = 0; k < j; k++) d -= A[j * n + k] * A[j * n + k];
    if (!(d > 0)) return false;
    d = std::sqrt(d);
    A[j * n + j] = d;
    for (int i = j + 1; i < n; i++) {
      S s = A[i * n + j];
      for (int k = 0; k < j; k++) s -= A[i * n + k] * A[j * n + k];
      A[i * n + j] = s / d;
    }
  }
  for (int i = 0; i < n; i++) {
    S s = b[i];
    for (int k = 0; k < i; k++) s -= A[i * n + k] * b[k];
    b[i] = s / A[i * n + i];
  }
  for (int i = n - 1; i >= 0; i--) {
    S s = b[i];
    for (int k = i + 1; k < n; k++) s -= A[k * n + i] * b[k];
    b[i] = s / A[i * n + i];
  }
  return true;
}
template <class S> bool inv_small(int n, const S* A, S* Ainv) {  // Gauss-Jordan, partial pivoting
  std::vector<S> M(A, A + n * n), I(n * n, S(0));
  for (int i = 0; i < n; i++) I[i * n + i] = 1;
  for (int c = 0; c < n; c++) {
    int piv = c;
    for (int r = c + 1; r < n; r++)
      if (std::fabs(M[r * n + c]) > std::fabs(M[piv * n + c])) piv = r;
    if (M[piv * n + c] == 0) return false;
    for (int k = 0; k < n; k++) {
      std::swap(M[c * n + k], M[piv * n + k]);
      std::swap(I[c * n + k], I[piv * n + k]);
    }
    S d = M[c * n + c];
    for (int k = 0; k < n; k++) { M[c * n + k] /= d; I[c * n + k] /= d; }
    for (int r = 0; r < n; r++)
      if (r != c) {
        S f = M[r * n + c];
        if (f != 0)
          for (int k = 0; k < n; k++) { M[r * n + k] -= f * M[c * n + k]; I[r * n + k] -= f * I[c * n + k]; }
      }
  }
  for (int i = 0; i < n * n; i++) Ainv[i] = I[i];
  return true;
}

// ---- model -----------------------------------------------------------------
struct Model {
  int nj = 0, nq = 0, nv = 0, nq_ext = 0;
  std::vector<int> parent, type, idx_q, idx_v, nqj, nvj;
  std::vector<V3<double>> axis;
  std::vector<SE3<double>> placement;
  std::vector<M6<double>> I6;
  V3<double> gravity{0, 0, -9.81};
  std::vector<int> ext_joints, ext_qoff, ext_voff, s2p;  // s2p[k] = internal v index of ext dof k
  std::vector<int> link_joint;
  std::vector<SE3<double>> link_placement;
  bool long_double = false;
};

template <class S> SE3<S> cast(const SE3<double>& m) {
  SE3<S> r;
  for (int i = 0; i < 9; i++) r.R[i] = S(m.R[i]);
  for (int i = 0; i < 3; i++) r.p[i] = S(m.p[i]);
  return r;
}
template <class S> M6<S> cast6(const M6<double>& m) {
  M6<S> r;
  for (int i = 0; i < 36; i++) r[i] = S(m[i]);
  return r;
}

// Joint transform and motion subspace (6 x nv_j, column-major in S6[c*6 + r]).
template <class S> SE3<S> jcalc(const Model& m, int i, const S* qint, S* S6) {
  SE3<S> M = se3id<S>();
  V3<S> a{S(m.axis[i][0]), S(m.axis[i][1]), S(m.axis[i][2])};
  const S* q = qint + m.idx_q[i];
  switch (m.type[i]) {
    case JT_REVOLUTE:
      M.R = rodrigues(a, S(std::sin(q[0])), S(std::cos(q[0])));
      for (int r = 0; r < 6; r++) S6[r] = r >= 3 ? a[r - 3] : S(0);
      break;
    case JT_CONTINUOUS:
      M.R = rodrigues(a, q[1], q[0]);
      for (int r = 0; r < 6; r++) S6[r] = r >= 3 ? a[r - 3] : S(0);
      break;
    case JT_PRISMATIC:
      for (int k = 0; k < 3; k++) M.p[k] = a[k] * q[0];
      for (int r = 0; r < 6; r++) S6[r] = r < 3 ? a[r] : S(0);
      break;
    case JT_FREEFLYER:
      M.p = {q[0], q[1], q[2]};
      M.R = quat_to_R(q[3], q[4], q[5], q[6]);
      for (int c = 0; c < 6; c++)
        for (int r = 0; r < 6; r++) S6[c * 6 + r] = (r == c) ? S(1) : S(0);
      break;
    default:
      break;
  }
  return M;
}

// posS2P: external q (joint-ordered; 1 value per 1-DoF joint, 7 per free flyer)
// -> internal configuration (cos/sin pair for unbounded revolute joints).
template <class S> void pos_s2p(const Model& m, const double* qe, S* qi) {
  for (size_t n = 0; n < m.ext_joints.size(); n++) {
    int j = m.ext_joints[n], o = m.ext_qoff[n], iq = m.idx_q[j];
    switch (m.type[j]) {
      case JT_CONTINUOUS:
        qi[iq] = S(std::cos(qe[o]));
        qi[iq + 1] = S(std::sin(qe[o]));
        break;
      case JT_FREEFLYER:
        for (int k = 0; k < 7; k++) qi[iq + k] = S(qe[o + k]);
        break;
      default:
        qi[iq] = S(qe[o]);
    }
  }
}
template <class S> void pos_p2s(const Model& m, const S* qi, double* qe) {
  for (size_t n = 0; n < m.ext_joints.size(); n++) {
    int j = m.ext_joints[n], o = m.ext_qoff[n], iq = m.idx_q[j];
    switch (m.type[j]) {
      case JT_CONTINUOUS: qe[o] = double(std::atan2(qi[iq + 1], qi[iq])); break;
      case JT_FREEFLYER:
        for (int k = 0; k < 7; k++) qe[o + k] = double(qi[iq + k]);
        break;
      default: qe[o] = double(qi[iq]);
    }
  }
}
template <class S> void vel_s2p(const Model& m, const double* ve, S* vi) {
  for (int k = 0; k < m.nv; k++) vi[m.s2p[k]] = S(ve[k]);
}
template <class S> void vel_p2s(const Model& m, const S* vi, double* ve) {
  for (int k = 0; k < m.nv; k++) ve[k] = double(vi[m.s2p[k]]);
}

template <class S> struct Work {
  SE3<S> liMi[kMaxJ], oMi[kMaxJ];
  M6<S> X[kMaxJ];       // actinv(liMi): parent -> child motion transform
  S Sj[kMaxJ][36];      // motion subspaces
  V6<S> v[kMaxJ], a[kMaxJ], f[kMaxJ], c[kMaxJ], pA[kMaxJ];
  M6<S> IA[kMaxJ];
};

template <class S> void kinematics(const Model& m, const S* qi, Work<S>& w) {
  w.oMi[0] = se3id<S>();
  for (int i = 1; i < m.nj; i++) {
    SE3<S> MJ = jcalc(m, i, qi, w.Sj[i]);
    w.liMi[i] = se3mul(cast<S>(m.placement[i]), MJ);
    w.X[i] = actinv6(w.liMi[i]);
    w.oMi[i] = se3mul(w.oMi[m.parent[i]], w.liMi[i]);
  }
}

template <class S> void rnea_int(const Model& m, const S* qi, const S* vi, const S* ai, S* tau, Work<S>& w) {
  kinematics(m, qi, w);
  w.v[0] = V6<S>{};
  w.a[0] = V6<S>{S(-m.gravity[0]), S(-m.gravity[1]), S(-m.gravity[2]), 0, 0, 0};
  for (int i = 1; i < m.nj; i++) {
    int p = m.parent[i], nvi = m.nvj[i], iv = m.idx_v[i];
    V6<S> vJ{}, aJ{};
    for (int k = 0; k < nvi; k++)
      for (int r = 0; r < 6; r++) {
        vJ[r] += w.Sj[i][k * 6 + r] * vi[iv + k];
        aJ[r] += w.Sj[i][k * 6 + r] * ai[iv + k];
      }
    w.v[i] = addv6(mv6(w.X[i], w.v[p]), vJ);
    w.a[i] = addv6(addv6(mv6(w.X[i], w.a[p]), aJ), mv6(crm(w.v[i]), vJ));
    M6<S> I = cast6<S>(m.I6[i]);
    w.f[i] = addv6(mv6(I, w.a[i]), mv6(crf(w.v[i]), mv6(I, w.v[i])));
  }
  for (int i = m.nj - 1; i >= 1; i--) {
    int p = m.parent[i], nvi = m.nvj[i], iv = m.idx_v[i];
    for (int k = 0; k < nvi; k++) {
      S s = 0;
      for (int r = 0; r < 6; r++) s += w.Sj[i][k * 6 + r] * w.f[i][r];
      tau[iv + k] = s;
    }
    if (p > 0) w.f[p] = addv6(w.f[p], mv6(tr6(w.X[i]), w.f[i]));
  }
}

template <class S> bool aba_int(const Model& m, const S* qi, const S* vi, const S* taui, S* qdd, Work<S>& w) {
  kinematics(m, qi, w);
  w.v[0] = V6<S>{};
  static thread_local std::vector<S> Ustore, Dinvstore, ustore;
  Ustore.assign(size_t(m.nv) * 6, S(0));
  Dinvstore.assign(size_t(m.nv) * 6, S(0));
  ustore.assign(size_t(m.nv), S(0));
  for (int i = 1; i < m.nj; i++) {
    int p = m.parent[i], nvi = m.nvj[i], iv = m.idx_v[i];
    V6<S> vJ{};
    for (int k = 0; k < nvi; k++)
      for (int r = 0; r < 6; r++) vJ[r] += w.Sj[i][k * 6 + r] * vi[iv + k];
    w.v[i] = addv6(mv6(w.X[i], w.v[p]), vJ);
    w.c[i] = mv6(crm(w.v[i]), vJ);
    w.IA[i] = cast6<S>(m.I6[i]);
    w.pA[i] = mv6(crf(w.v[i]), mv6(w.IA[i], w.v[i]));
  }
  for (int i = m.nj - 1; i >= 1; i--) {
    int p = m.parent[i], nvi = m.nvj[i], iv = m.idx_v[i];
    // U = IA S (6 x nvi), D = S^T U, u = tau - S^T pA
    S U[36], D[36], Dinv[36], u[6];
    for (int k = 0; k < nvi; k++)
      for (int r = 0; r < 6; r++) {
        S s = 0;
        for (int c = 0; c < 6; c++) s += w.IA[i][r * 6 + c] * w.Sj[i][k * 6 + c];
        U[k * 6 + r] = s;
      }
    for (int k = 0; k < nvi; k++) {
      for (int l = 0; l < nvi; l++) {
        S s = 0;
        for (int r = 0; r < 6; r++) s += w.Sj[i][k * 6 + r] * U[l * 6 + r];
        D[k * nvi + l] = s;
      }
      S s = 0;
      for (int r = 0; r < 6; r++) s += w.Sj[i][k * 6 + r] * w.pA[i][r];
      u[k] = taui[iv + k] - s;
    }
    if (!inv_small(nvi, D, Dinv)) return false;
    for (int k = 0; k < nvi * 6; k++) Ustore[size_t(iv) * 6 + k] = U[k];
    for (int k = 0; k < nvi * nvi; k++) Dinvstore[size_t(iv) * 6 + k] = Dinv[k];
    for (int k = 0; k < nvi; k++) ustore[iv + k] = u[k];
    if (p > 0) {
      // Ia = IA - U Dinv U^T ; pa = pA + Ia c + U Dinv u
      M6<S> Ia = w.IA[i];
      S UD[36];  // U Dinv (6 x nvi)
      for (int k = 0; k < nvi; k++)
        for (int r = 0; r < 6; r++) {
          S s = 0;
          for (int l = 0; l < nvi; l++) s += U[l * 6 + r] * Dinv[l * nvi + k];
          UD[k * 6 + r] = s;
        }
      for (int r = 0; r < 6; r++)
        for (int c = 0; c < 6; c++) {
          S s = 0;
          for (int k = 0; k < nvi; k++) s += UD[k * 6 + r] * U[k * 6 + c];
          Ia[r * 6 + c] -= s;
        }
      V6<S> pa = addv6(w.pA[i], mv6(Ia, w.c[i]));
      for (int r = 0; r < 6; r++) {
        S s = 0;
        for (int k = 0; k < nvi; k++) s += UD[k * 6 + r] * u[k];
        pa[r] += s;
      }
      M6<S> XT = tr6(w.X[i]);
      M6<S> contrib = mul6(mul6(XT, Ia), w.X[i]);
      for (int k = 0; k < 36; k++) w.IA[p][k] += contrib[k];
      w.pA[p] = addv6(w.pA[p], mv6(XT, pa));
    }
  }
  w.a[0] = V6<S>{S(-m.gravity[0]), S(-m.gravity[1]), S(-m.gravity[2]), 0, 0, 0};
  for (int i = 1; i < m.nj; i++) {
    int p = m.parent[i], nvi = m.nvj[i], iv = m.idx_v[i];
    V6<S> ap = addv6(mv6(w.X[i], w.a[p]), w.c[i]);
    S rhs[6];
    for (int k = 0; k < nvi; k++) {
      S s = 0;
      for (int r = 0; r < 6; r++) s += Ustore[size_t(iv) * 6 + k * 6 + r] * ap[r];
      rhs[k] = ustore[iv + k] - s;
    }
    for (int k = 0; k < nvi; k++) {
      S s = 0;
      for (int l = 0; l < nvi; l++) s += Dinvstore[size_t(iv) * 6 + k * nvi + l] * rhs[l];
      qdd[iv + k] = s;
    }
    for (int k = 0; k < nvi; k++)
      for (int r = 0; r < 6; r++) ap[r] += w.Sj[i][k * 6 + r] * qdd[iv + k];
    w.a[i] = ap;
  }
  return true;
}

// Composite-rigid-body mass matrix (upper triangle filled, then mirrored).
template <class S> void crba_int(const Model& m, const S* qi, S* M, Work<S>& w) {
  kinematics(m, qi, w);
  int nv = m.nv;
  for (int k = 0; k < nv * nv; k++) M[k] = 0;
  for (int i = 1; i < m.nj; i++) w.IA[i] = cast6<S>(m.I6[i]);
  for (int i = m.nj - 1; i >= 1; i--) {
    int p = m.parent[i];
    if (p > 0) {
      M6<S> contrib = mul6(mul6(tr6(w.X[i]), w.IA[i]), w.X[i]);
      for (int k = 0; k < 36; k++) w.IA[p][k] += contrib[k];
    }
  }
  for (int i = 1; i < m.nj; i++) {
    int nvi = m.nvj[i], iv = m.idx_v[i];
    for (int k = 0; k < nvi; k++) {
      V6<S> col;
      for (int r = 0; r < 6; r++) col[r] = w.Sj[i][k * 6 + r];
      V6<S> F = mv6(w.IA[i], col);
      int j = i;
      while (j > 0) {
        int jv = m.idx_v[j];
        for (int l = 0; l < m.nvj[j]; l++) {
          S s = 0;
          for (int r = 0; r < 6; r++) s += w.Sj[j][l * 6 + r] * F[r];
          if (jv + l <= iv + k) M[(jv + l) * nv + iv + k] = s;  // upper triangle
        }
        if (m.parent[j] > 0) F = mv6(tr6(w.X[j]), F);
        j = m.parent[j];
      }
    }
  }
  for (int r = 0; r < nv; r++)
    for (int c = 0; c < r; c++) M[r * nv + c] = M[c * nv + r];
}

// WORLD Jacobian (6 x nv, row-major) of all joints: column = oMi.act(S).
template <class S> void jac_world(const Model& m, const Work<S>& w, S* J) {
  int nv = m.nv;
  for (int i = 1; i < m.nj; i++) {
    M6<S> A = act6(w.oMi[i]);
    for (int k = 0; k < m.nvj[i]; k++) {
      V6<S> col;
      for (int r = 0; r < 6; r++) col[r] = w.Sj[i][k * 6 + r];
      V6<S> o = mv6(A, col);
      for (int r = 0; r < 6; r++) J[r * nv + m.idx_v[i] + k] = o[r];
    }
  }
}
template <class S> std::vector<char> support_mask(const Model& m, int joint) {
  std::vector<char> in(m.nv, 0);
  for (int j = joint; j > 0; j = m.parent[j])
    for (int k = 0; k < m.nvj[j]; k++) in[m.idx_v[j] + k] = 1;
  return in;
}

// Christoffel-consistent Coriolis matrix, world frame:
// C = sum_i J_i^T (I_i Jdot_i + B(I_i, v_i) J_i), B = 1/2 (v x* I - I v x + (I v) xbar*).
template <class S> void coriolis_int(const Model& m, const S* qi, const S* vi, S* C, Work<S>& w) {
  kinematics(m, qi, w);
  int nv = m.nv;
  std::vector<S> J(6 * nv, S(0));
  jac_world(m, w, J.data());
  // world spatial velocity of each body
  std::vector<V6<S>> vw(m.nj);
  vw[0] = V6<S>{};
  for (int i = 1; i < m.nj; i++) {
    V6<S> s = vw[m.parent[i]];
    for (int k = 0; k < m.nvj[i]; k++)
      for (int r = 0; r < 6; r++) s[r] += J[r * nv + m.idx_v[i] + k] * vi[m.idx_v[i] + k];
    vw[i] = s;
  }
  // Jdot columns: d/dt (oMi.act S) = v_i x (oMi.act S)
  std::vector<S> Jd(6 * nv, S(0));
  for (int i = 1; i < m.nj; i++)
    for (int k = 0; k < m.nvj[i]; k++) {
      V6<S> col;
      for (int r = 0; r < 6; r++) col[r] = J[r * nv + m.idx_v[i] + k];
      V6<S> d = mv6(crm(vw[i]), col);
      for (int r = 0; r < 6; r++) Jd[r * nv + m.idx_v[i] + k] = d[r];
    }
  for (int k = 0; k < nv * nv; k++) C[k] = 0;
  for (int i = 1; i < m.nj; i++) {
    M6<S> Af = tr6(actinv6(w.oMi[i]));  // force transform body -> world
    M6<S> Iw = mul6(mul6(Af, cast6<S>(m.I6[i])), actinv6(w.oMi[i]));
    V6<S> h = mv6(Iw, vw[i]);
    // (h xbar*) : matrix with (h xbar*) v = v x* h
    M6<S> Hb{};
    for (int c = 0; c < 6; c++) {
      V6<S> e{};
      e[c] = 1;
      V6<S> col = mv6(crf(e), h);
      for (int r = 0; r < 6; r++) Hb[r * 6 + c] = col[r];
    }
    M6<S> B = mul6(crf(vw[i]), Iw);
    M6<S> IV = mul6(Iw, crm(vw[i]));
    for (int k = 0; k < 36; k++) B[k] = S(0.5) * (B[k] - IV[k] + Hb[k]);
    auto in = support_mask<S>(m, i);
    for (int l = 0; l < nv; l++) {
      if (!in[l]) continue;
      V6<S> jl, jdl;
      for (int r = 0; r < 6; r++) { jl[r] = J[r * nv + l]; jdl[r] = Jd[r * nv + l]; }
      V6<S> F = addv6(mv6(Iw, jdl), mv6(B, jl));
      for (int kk = 0; kk < nv; kk++) {
        if (!in[kk]) continue;
        S s = 0;
        for (int r = 0; r < 6; r++) s += J[r * nv + kk] * F[r];
        C[kk * nv + l] += s;
      }
    }
  }
}

template <class S> void neutral(const Model& m, S* qi) {
  for (int j = 1; j < m.nj; j++) {
    int iq = m.idx_q[j];
    switch (m.type[j]) {
      case JT_CONTINUOUS: qi[iq] = 1; qi[iq + 1] = 0; break;
      case JT_FREEFLYER:
        for (int k = 0; k < 7; k++) qi[iq + k] = (k == 6) ? 1 : 0;
        break;
      default: qi[iq] = 0;
    }
  }
}
// Internal-configuration integrator q (+) v.
template <class S> void integrate_int(const Model& m, const S* q, const S* v, S* out) {
  for (int j = 1; j < m.nj; j++) {
    int iq = m.idx_q[j], iv = m.idx_v[j];
    switch (m.type[j]) {
      case JT_CONTINUOUS: {
        // multiply the unit complex number (c, s) by exp(i v), then a first-order
        // renormalisation z <- z (3 - |z|^2) / 2
        S c = q[iq], s = q[iq + 1], cw = std::cos(v[iv]), sw = std::sin(v[iv]);
        S nc = cw * c - sw * s, ns = sw * c + cw * s;
        S k = (3 - (nc * nc + ns * ns)) / 2;
        out[iq] = nc * k;
        out[iq + 1] = ns * k;
        break;
      }
      case JT_FREEFLYER: {
        SE3<S> M0;
        M0.p = {q[iq], q[iq + 1], q[iq + 2]};
        M0.R = quat_to_R(q[iq + 3], q[iq + 4], q[iq + 5], q[iq + 6]);
        V6<S> nu;
        for (int k = 0; k < 6; k++) nu[k] = v[iv + k];
        SE3<S> M1 = se3mul(M0, exp6(nu));
        auto qw = R_to_quat(M1.R);  // w x y z
        S dotq = qw[1] * q[iq + 3] + qw[2] * q[iq + 4] + qw[3] * q[iq + 5] + qw[0] * q[iq + 6];
        if (dotq < 0) for (auto& x : qw) x = -x;
        S n = std::sqrt(qw[0] * qw[0] + qw[1] * qw[1] + qw[2] * qw[2] + qw[3] * qw[3]);
        for (int k = 0; k < 3; k++) out[iq + k] = M1.p[k];
        out[iq + 3] = qw[1] / n;
        out[iq + 4] = qw[2] / n;
        out[iq + 5] = qw[3] / n;
        out[iq + 6] = qw[0] / n;
        break;
      }
      default: out[iq] = q[iq] + v[iv];
    }
  }
}

// computeJointJacobian: Jacobian of joint `jid` expressed in its own frame.
template <class S> void joint_jacobian_local(const Model& m, const Work<S>& w, int jid, S* J) {
  int nv = m.nv;
  for (int k = 0; k < 6 * nv; k++) J[k] = 0;
  M6<S> Ainv = actinv6(w.oMi[jid]);
  for (int j = jid; j > 0; j = m.parent[j]) {
    M6<S> A = mul6(Ainv, act6(w.oMi[j]));
    for (int k = 0; k < m.nvj[j]; k++) {
      V6<S> col;
      for (int r = 0; r < 6; r++) col[r] = w.Sj[j][k * 6 + r];
      V6<S> o = mv6(A, col);
      for (int r = 0; r < 6; r++) J[r * nv + m.idx_v[j] + k] = o[r];
    }
  }
}

struct Handle {
  Model m;
  // cached by orc_full_jacobian for orc_link_jacobian (like Pinocchio Data)
  std::vector<double> J;
  std::vector<SE3<double>> oMi;
};

template <class S> void fk_poses(const Model& m, const double* qe, double* out /* nlinks x 12 */) {
  S qi[kMaxV];
  pos_s2p(m, qe, qi);
  static thread_local Work<S> w;
  kinematics(m, qi, w);
  for (size_t l = 0; l < m.link_joint.size(); l++) {
    SE3<S> T = se3mul(w.oMi[m.link_joint[l]], cast<S>(m.link_placement[l]));
    for (int k = 0; k < 9; k++) out[l * 12 + k] = double(T.R[k]);
    for (int k = 0; k < 3; k++) out[l * 12 + 9 + k] = double(T.p[k]);
  }
}

template <class S> int rnea_ext(const Model& m, const double* q, const double* qd, const double* qdd, double* tau) {
  S qi[kMaxV], vi[kMaxV], ai[kMaxV], ti[kMaxV];
  pos_s2p(m, q, qi);
  vel_s2p(m, qd, vi);
  vel_s2p(m, qdd, ai);
  static thread_local Work<S> w;
  rnea_int(m, qi, vi, ai, ti, w);
  vel_p2s(m, ti, tau);
  return 0;
}
template <class S> int aba_ext(const Model& m, const double* q, const double* qd, const double* tau, double* qdd) {
  S qi[kMaxV], vi[kMaxV], ti[kMaxV], ai[kMaxV];
  pos_s2p(m, q, qi);
  vel_s2p(m, qd, vi);
  vel_s2p(m, tau, ti);
  static thread_local Work<S> w;
  if (!aba_int(m, qi, vi, ti, ai, w)) return -3;
  vel_p2s(m, ai, qdd);
  return 0;
}
template <class S> int crba_ext(const Model& m, const double* q, double* M) {
  S qi[kMaxV];
  pos_s2p(m, q, qi);
  static thread_local Work<S> w;
  std::vector<S> Mi(size_t(m.nv) * m.nv);
  crba_int(m, qi, Mi.data(), w);
  for (int r = 0; r < m.nv; r++)
    for (int c = 0; c < m.nv; c++) M[r * m.nv + c] = double(Mi[m.s2p[r] * m.nv + m.s2p[c]]);
  return 0;
}
template <class S> int coriolis_ext(const Model& m, const double* q, const double* qd, double* C) {
  S qi[kMaxV], vi[kMaxV];
  pos_s2p(m, q, qi);
  vel_s2p(m, qd, vi);
  static thread_local Work<S> w;
  std::vector<S> Ci(size_t(m.nv) * m.nv);
  coriolis_int(m, qi, vi, Ci.data(), w);
  for (int r = 0; r < m.nv; r++)
    for (int c = 0; c < m.nv; c++) C[r * m.nv + c] = double(Ci[m.s2p[r] * m.nv + m.s2p[c]]);
  return 0;
}
template <class S> void jac_full_ext(const Model& m, const double* q, double* Jout /* 6 x nv ext cols */) {
  S qi[kMaxV];
  pos_s2p(m, q, qi);
  static thread_local Work<S> w;
  kinematics(m, qi, w);
  std::vector<S> J(6 * size_t(m.nv), S(0));
  jac_world(m, w, J.data());
  for (int r = 0; r < 6; r++)
    for (int k = 0; k < m.nv; k++) Jout[r * m.nv + k] = double(J[r * m.nv + m.s2p[k]]);
}

template <class S> int ik_ext(const Model& m, int link, const double* target /*R9 p3*/, const double* q0,
                              const int* mask, double eps, int max_iter, double dt, double damp, double* q_out,
                              int* success, double* err_out) {
  int nv = m.nv;
  std::vector<S> q(m.nq), bestQ(m.nq), qn(m.nq), mk(nv, S(1));
  if (q0) pos_s2p(m, q0, q.data());
  else neutral(m, q.data());
  if (mask)
    for (int k = 0; k < nv; k++) mk[m.s2p[k]] = S(mask[k]);
  int jid = m.link_joint[link];
  SE3<S> l2w;
  for (int k = 0; k < 9; k++) l2w.R[k] = S(target[k]);
  for (int k = 0; k < 3; k++) l2w.p[k] = S(target[9 + k]);
  SE3<S> oMdes = se3mul(l2w, se3inv(cast<S>(m.link_placement[link])));
  std::vector<S> J(6 * size_t(nv)), v(nv);
  static thread_local Work<S> w;
  S minErr = S(1e10);
  bestQ = q;
  V6<S> bestErr{}, err;
  bool ok = false;
  for (int it = 0;; it++) {
    kinematics(m, q.data(), w);
    SE3<S> iMd = se3mul(se3inv(w.oMi[jid]), oMdes);
    err = log6(iMd);
    S n = 0;
    for (int k = 0; k < 6; k++) n += err[k] * err[k];
    n = std::sqrt(n);
    if (n < minErr) {
      minErr = n;
      bestQ = q;
      bestErr = err;
    }
    if (n < S(eps)) { ok = true; break; }
    if (it >= max_iter) { ok = false; break; }
    joint_jacobian_local(m, w, jid, J.data());
    M6<S> Jl = jlog6(se3inv(iMd));
    std::vector<S> J2(6 * size_t(nv));
    for (int r = 0; r < 6; r++)
      for (int c = 0; c < nv; c++) {
        S s = 0;
        for (int k = 0; k < 6; k++) s += Jl[r * 6 + k] * J[k * nv + c];
        J2[r * nv + c] = -s * mk[c];
      }
    std::vector<S> JJt(36);
    for (int r = 0; r < 6; r++)
      for (int c = 0; c < 6; c++) {
        S s = 0;
        for (int k = 0; k < nv; k++) s += J2[r * nv + k] * J2[c * nv + k];
        JJt[r * 6 + c] = s + (r == c ? S(damp) : S(0));
      }
    S x[6];
    for (int k = 0; k < 6; k++) x[k] = err[k];
    if (!chol_solve(6, JJt, x)) return -3;
    for (int c = 0; c < nv; c++) {
      S s = 0;
      for (int r = 0; r < 6; r++) s += J2[r * nv + c] * x[r];
      v[c] = -s * S(dt);
    }
    integrate_int(m, q.data(), v.data(), qn.data());
    q = qn;
  }
  pos_p2s(m, bestQ.data(), q_out);
  *success = ok ? 1 : 0;
  for (int k = 0; k < 6; k++) err_out[k] = double(bestErr[k]);
  return 0;
}

// External-coordinate integrator used by rollouts: angles and slides add, free
// flyers integrate on SE(3).
void integrate_ext(const Model& m, const double* q, const double* v, double* out) {
  for (size_t n = 0; n < m.ext_joints.size(); n++) {
    int j = m.ext_joints[n], o = m.ext_qoff[n], ov = m.ext_voff[n];
    if (m.type[j] == JT_FREEFLYER) {
      Model one;  // integrate a lone free flyer with the internal integrator
      one.nj = 2;
      one.type = {0, JT_FREEFLYER};
      one.idx_q = {0, 0};
      one.idx_v = {0, 0};
      integrate_int<double>(one, q + o, v + ov, out + o);
    } else {
      out[o] = q[o] + v[ov];
    }
  }
}

template <class F> void parallel_for(long n, int nthreads, F&& f) {
  if (nthreads <= 1 || n < 2) {
    for (long i = 0; i < n; i++) f(i);
    return;
  }
  std::vector<std::thread> th;
  long chunk = (n + nthreads - 1) / nthreads;
  for (int t = 0; t < nthreads; t++) {
    long b = t * chunk, e = std::min(n, b + chunk);
    if (b >= e) break;
    th.emplace_back([=, &f] {
      for (long i = b; i < e; i++) f(i);
    });
  }
  for (auto& x : th) x.join();
}

}  // namespace

extern "C" {

// Build from flat tables (joint 0 = universe). placement: nj x 12 (R row-major, p);
// inertia6: nj x 36; link_placement: nlinks x 12.
void* orc_create(int nj, const int* parent, const int* type, const double* axis, const double* placement,
                 const double* inertia6, const double* gravity, int n_ext, const int* ext_joints, int nlinks,
                 const int* link_joint, const double* link_placement) {
  if (nj > kMaxJ) return nullptr;
  auto* h = new Handle;
  Model& m = h->m;
  m.nj = nj;
  m.parent.assign(parent, parent + nj);
  m.type.assign(type, type + nj);
  m.axis.resize(nj);
  m.placement.resize(nj);
  m.I6.resize(nj);
  m.idx_q.resize(nj);
  m.idx_v.resize(nj);
  m.nqj.resize(nj);
  m.nvj.resize(nj);
  int nq = 0, nv = 0;
  for (int i = 0; i < nj; i++) {
    for (int k = 0; k < 3; k++) m.axis[i][k] = axis[i * 3 + k];
    for (int k = 0; k < 9; k++) m.placement[i].R[k] = placement[i * 12 + k];
    for (int k = 0; k < 3; k++) m.placement[i].p[k] = placement[i * 12 + 9 + k];
    for (int k = 0; k < 36; k++) m.I6[i][k] = inertia6[i * 36 + k];
    int tq = 0, tv = 0;
    switch (type[i]) {
      case JT_REVOLUTE: case JT_PRISMATIC: tq = 1; tv = 1; break;
      case JT_CONTINUOUS: tq = 2; tv = 1; break;
      case JT_FREEFLYER: tq = 7; tv = 6; break;
      default: break;
    }
    m.idx_q[i] = nq;
    m.idx_v[i] = nv;
    m.nqj[i] = tq;
    m.nvj[i] = tv;
    nq += tq;
    nv += tv;
  }
  m.nq = nq;
  m.nv = nv;
  if (nv > kMaxV) { delete h; return nullptr; }
  for (int k = 0; k < 3; k++) m.gravity[k] = gravity[k];
  m.ext_joints.assign(ext_joints, ext_joints + n_ext);
  int qo = 0, vo = 0;
  for (int n = 0; n < n_ext; n++) {
    int j = ext_joints[n];
    m.ext_qoff.push_back(qo);
    m.ext_voff.push_back(vo);
    qo += (m.type[j] == JT_FREEFLYER) ? 7 : 1;
    for (int k = 0; k < m.nvj[j]; k++) m.s2p.push_back(m.idx_v[j] + k);
    vo += m.nvj[j];
  }
  m.nq_ext = qo;
  if (vo != nv) { delete h; return nullptr; }
  m.link_joint.assign(link_joint, link_joint + nlinks);
  m.link_placement.resize(nlinks);
  for (int l = 0; l < nlinks; l++) {
    for (int k = 0; k < 9; k++) m.link_placement[l].R[k] = link_placement[l * 12 + k];
    for (int k = 0; k < 3; k++) m.link_placement[l].p[k] = link_placement[l * 12 + 9 + k];
  }
  return h;
}
void orc_free(void* h) { delete static_cast<Handle*>(h); }
void orc_set_long_double(void* h, int on) { static_cast<Handle*>(h)->m.long_double = on != 0; }
int orc_info(void* h, int* nq, int* nv, int* nq_ext) {
  auto& m = static_cast<Handle*>(h)->m;
  *nq = m.nq;
  *nv = m.nv;
  *nq_ext = m.nq_ext;
  return 0;
}

#define DISPATCH(call_d, call_ld) (m.long_double ? (call_ld) : (call_d))

int orc_fk(void* hh, const double* q, double* out) {
  auto& m = static_cast<Handle*>(hh)->m;
  if (m.long_double) fk_poses<long double>(m, q, out);
  else fk_poses<double>(m, q, out);
  return 0;
}
int orc_rnea(void* hh, const double* q, const double* qd, const double* qdd, double* tau) {
  auto& m = static_cast<Handle*>(hh)->m;
  return DISPATCH(rnea_ext<double>(m, q, qd, qdd, tau), rnea_ext<long double>(m, q, qd, qdd, tau));
}
int orc_aba(void* hh, const double* q, const double* qd, const double* tau, double* qdd) {
  auto& m = static_cast<Handle*>(hh)->m;
  return DISPATCH(aba_ext<double>(m, q, qd, tau, qdd), aba_ext<long double>(m, q, qd, tau, qdd));
}
int orc_crba(void* hh, const double* q, double* M) {
  auto& m = static_cast<Handle*>(hh)->m;
  return DISPATCH(crba_ext<double>(m, q, M), crba_ext<long double>(m, q, M));
}
int orc_coriolis(void* hh, const double* q, const double* qd, double* C) {
  auto& m = static_cast<Handle*>(hh)->m;
  return DISPATCH(coriolis_ext<double>(m, q, qd, C), coriolis_ext<long double>(m, q, qd, C));
}
// computeFullJacobian: caches the WORLD Jacobian and joint placements.
int orc_full_jacobian(void* hh, const double* q, double* Jout /* may be null; 6 x nv, ext columns */) {
  auto* h = static_cast<Handle*>(hh);
  auto& m = h->m;
  double qi[kMaxV];
  pos_s2p(m, q, qi);
  static thread_local Work<double> w;
  kinematics(m, qi, w);
  h->J.assign(6 * size_t(m.nv), 0.0);
  jac_world(m, w, h->J.data());
  h->oMi.assign(w.oMi, w.oMi + m.nj);
  if (Jout)
    for (int r = 0; r < 6; r++)
      for (int k = 0; k < m.nv; k++) Jout[r * m.nv + k] = h->J[r * m.nv + m.s2p[k]];
  return 0;
}
// getLinkJacobian after orc_full_jacobian; local != 0 -> link (body) frame.
int orc_link_jacobian(void* hh, int link, int local, double* out) {
  auto* h = static_cast<Handle*>(hh);
  auto& m = h->m;
  if (link < 0 || link >= int(m.link_joint.size())) return -2;
  if (h->J.empty()) return -4;
  int jid = m.link_joint[link], nv = m.nv;
  auto in = support_mask<double>(m, jid);
  std::vector<double> J(6 * size_t(nv), 0.0);
  for (int r = 0; r < 6; r++)
    for (int c = 0; c < nv; c++)
      if (in[c]) J[r * nv + c] = h->J[r * nv + c];
  if (local) {
    SE3<double> l2w = se3mul(h->oMi[jid], m.link_placement[link]);
    M6<double> A = actinv6(l2w);
    std::vector<double> J2(6 * size_t(nv));
    for (int r = 0; r < 6; r++)
      for (int c = 0; c < nv; c++) {
        double s = 0;
        for (int k = 0; k < 6; k++) s += A[r * 6 + k] * J[k * nv + c];
        J2[r * nv + c] = s;
      }
    J = J2;
  }
  for (int r = 0; r < 6; r++)
    for (int k = 0; k < nv; k++) out[r * nv + k] = J[r * nv + m.s2p[k]];
  return 0;
}
int orc_single_link_local_jacobian(void* hh, const double* q, int link, double* out) {
  auto& m = static_cast<Handle*>(hh)->m;
  if (link < 0 || link >= int(m.link_joint.size())) return -2;
  double qi[kMaxV];
  pos_s2p(m, q, qi);
  static thread_local Work<double> w;
  kinematics(m, qi, w);
  int nv = m.nv, jid = m.link_joint[link];
  std::vector<double> J(6 * size_t(nv));
  joint_jacobian_local(m, w, jid, J.data());
  M6<double> A = actinv6(m.link_placement[link]);
  for (int r = 0; r < 6; r++)
    for (int k = 0; k < nv; k++) {
      double s = 0;
      for (int t = 0; t < 6; t++) s += A[r * 6 + t] * J[t * nv + m.s2p[k]];
      out[r * nv + k] = s;
    }
  return 0;
}
int orc_ik(void* hh, int link, const double* target, const double* q0, const int* mask, double eps, int max_iter,
           double dt, double damp, double* q_out, int* success, double* err6) {
  auto& m = static_cast<Handle*>(hh)->m;
  if (link < 0 || link >= int(m.link_joint.size())) return -2;
  return DISPATCH(ik_ext<double>(m, link, target, q0, mask, eps, max_iter, dt, damp, q_out, success, err6),
                  ik_ext<long double>(m, link, target, q0, mask, eps, max_iter, dt, damp, q_out, success, err6));
}
int orc_integrate(void* hh, const double* q, const double* v, double* out) {
  integrate_ext(static_cast<Handle*>(hh)->m, q, v, out);
  return 0;
}
int orc_neutral(void* hh, double* q_ext) {
  auto& m = static_cast<Handle*>(hh)->m;
  double qi[kMaxV];
  neutral(m, qi);
  pos_p2s(m, qi, q_ext);
  return 0;
}
// SE(3) helpers exposed for identity tests: M as R9 p3.
void orc_log6(const double* M12, double* out6) {
  SE3<double> M;
  for (int k = 0; k < 9; k++) M.R[k] = M12[k];
  for (int k = 0; k < 3; k++) M.p[k] = M12[9 + k];
  auto v = log6(M);
  for (int k = 0; k < 6; k++) out6[k] = v[k];
}
void orc_exp6(const double* nu6, double* M12) {
  V6<double> nu;
  for (int k = 0; k < 6; k++) nu[k] = nu6[k];
  auto M = exp6(nu);
  for (int k = 0; k < 9; k++) M12[k] = M.R[k];
  for (int k = 0; k < 3; k++) M12[9 + k] = M.p[k];
}
void orc_jlog6(const double* M12, double* out36) {
  SE3<double> M;
  for (int k = 0; k < 9; k++) M.R[k] = M12[k];
  for (int k = 0; k < 3; k++) M.p[k] = M12[9 + k];
  auto J = jlog6(M);
  for (int k = 0; k < 36; k++) out36[k] = J[k];
}

// ---- operation counts ----------------------------------------------------------------
// Runs each of forward kinematics (link poses), the full WORLD Jacobian, CRBA, RNEA and ABA
// once on the counting scalar and writes, per op, {add, mul, div, sqrt, trig} to
// counts[op * 5 + k] (op 0..4 in that order); op 5 is the shared joint-placement pass
// (posS2P + forward kinematics of the joints) that every one of them starts with.
int orc_count_ops(void* hh, const double* q, const double* qd, const double* qdd, const double* tau,
                  long long* counts) {
  using orc_count::Cnt;
  using orc_count::g_counts;
  auto& m = static_cast<Handle*>(hh)->m;
  const int nv = m.nv, nl = int(m.link_joint.size());
  std::vector<double> poses(size_t(nl) * 12), J(6 * size_t(nv)), M(size_t(nv) * nv), t(nv), a(nv);
  auto record = [&](int op) {
    const long long v[5] = {g_counts.add, g_counts.mul, g_counts.div, g_counts.sqrt, g_counts.trig};
    for (int k = 0; k < 5; k++) counts[op * 5 + k] = v[k];
    g_counts = orc_count::Counts{};
  };
  g_counts = orc_count::Counts{};
  fk_poses<Cnt>(m, q, poses.data());
  record(0);
  jac_full_ext<Cnt>(m, q, J.data());
  record(1);
  crba_ext<Cnt>(m, q, M.data());
  record(2);
  rnea_ext<Cnt>(m, q, qd, qdd, t.data());
  record(3);
  if (aba_ext<Cnt>(m, q, qd, tau, a.data()) != 0) return -3;
  record(4);
  {
    Cnt qi[kMaxV];
    pos_s2p(m, q, qi);
    static thread_local Work<Cnt> w;
    kinematics(m, qi, w);
  }
  record(5);
  return 0;
}

// ---- batched drivers (per-environment single-instance calls, threads over envs) ----
// Arrays are row-major [n][cols]. ops bitmask for orc_batch_step: 1 FK poses, 2 full
// Jacobian, 4 CRBA, 8 RNEA, 16 ABA.
int orc_batch_step(void* hh, long n, int ops, const double* q, const double* qd, const double* qdd,
                   const double* tau, double* poses, double* J, double* M, double* tau_out, double* qdd_out,
                   int nthreads) {
  auto& m = static_cast<Handle*>(hh)->m;
  const long nqe = m.nq_ext, nv = m.nv, nl = long(m.link_joint.size());
  parallel_for(n, nthreads, [&](long e) {
    const double* qe = q + e * nqe;
    if (ops & 1) fk_poses<double>(m, qe, poses + e * nl * 12);
    if (ops & 2) jac_full_ext<double>(m, qe, J + e * 6 * nv);
    if (ops & 4) crba_ext<double>(m, qe, M + e * nv * nv);
    if (ops & 8) rnea_ext<double>(m, qe, qd + e * nv, qdd + e * nv, tau_out + e * nv);
    if (ops & 16) aba_ext<double>(m, qe, qd + e * nv, tau + e * nv, qdd_out + e * nv);
  });
  return 0;
}
int orc_batch_ik(void* hh, long n, int link, const double* targets /* n x 12 */, const double* q0 /* n x nqe or null */,
                 double eps, int max_iter, double dt, double damp, double* q_out, int* success, double* err6,
                 int nthreads) {
  auto& m = static_cast<Handle*>(hh)->m;
  const long nqe = m.nq_ext;
  parallel_for(n, nthreads, [&](long e) {
    ik_ext<double>(m, link, targets + e * 12, q0 ? q0 + e * nqe : nullptr, nullptr, eps, max_iter, dt, damp,
                   q_out + e * nqe, success + e, err6 + e * 6);
  });
  return 0;
}
// Semi-implicit Euler rollout: qd += dt ABA(q, qd, tau_t); q = q (+) dt qd.
// tau: [T][n][nv]. Loss per env: |p_link(q_T) - target|^2.
int orc_rollout(void* hh, long n, int T, double dt, const double* q0, const double* qd0, const double* tau,
                int link, const double* targets /* n x 3 */, double* qT, double* qdT, double* loss, int nthreads) {
  auto& m = static_cast<Handle*>(hh)->m;
  const long nqe = m.nq_ext, nv = m.nv, nl = long(m.link_joint.size());
  parallel_for(n, nthreads, [&](long e) {
    std::vector<double> q(q0 + e * nqe, q0 + (e + 1) * nqe), qd(qd0 + e * nv, qd0 + (e + 1) * nv), a(nv), dq(nv),
        qn(nqe), poses(nl * 12);
    for (int t = 0; t < T; t++) {
      aba_ext<double>(m, q.data(), qd.data(), tau + (size_t(t) * n + e) * nv, a.data());
      for (long k = 0; k < nv; k++) {
        qd[k] += dt * a[k];
        dq[k] = dt * qd[k];
      }
      integrate_ext(m, q.data(), dq.data(), qn.data());
      q = qn;
    }
    for (long k = 0; k < nqe; k++) qT[e * nqe + k] = q[k];
    for (long k = 0; k < nv; k++) qdT[e * nv + k] = qd[k];
    fk_poses<double>(m, q.data(), poses.data());
    double s = 0;
    for (int k = 0; k < 3; k++) {
      double d = poses[link * 12 + 9 + k] - targets[e * 3 + k];
      s += d * d;
    }
    loss[e] = s;
  });
  return 0;
}

}  // extern "C"
