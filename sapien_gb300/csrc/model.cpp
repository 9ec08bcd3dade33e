// URDF -> kinematic tree with the conventions of pinocchio::urdf::buildModelFromXML
// (reached from pinocchio/pinocchio_model.cpp:42). The semantics restated here:
//  * the root link is welded to the universe joint 0 (fromURDFXML passes no root joint);
//  * links are visited depth first, the children of a link in byte-wise order of their
//    joint names (urdfdom stores joints in a std::map keyed by name);
//  * a moving joint's placement is parent_body_frame.placement * origin, relative to the
//    moving joint carrying the parent link; the child link's inertia is attached to it;
//  * a fixed joint adds no DoF: the child's inertia is transported by
//    parent_body_frame.placement * origin and added to the carrying joint, and the
//    child's BODY frame gets that placement;
//  * revolute (nq 1), continuous (nq 2 internally as cos/sin, one external angle),
//    prismatic (nq 1), floating (free flyer x y z qx qy qz qw, nv 6);
//  * link inertials: com = origin.xyz, rotational inertia R(origin.rpy) I R^T;
//  * rpy -> rotation through the half-angle quaternion.
// setJointOrder / setLinkOrder follow pinocchio/pinocchio_model.cpp:99-140.
#include "model.h"

#include <random>

#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <charconv>
#include <cmath>
#include <cstring>
#include <functional>
#include <set>
#include <stdexcept>

#include "xml.h"

namespace sgdyn {
namespace {

struct InvalidArgument : std::invalid_argument {
  using std::invalid_argument::invalid_argument;
};

void parse_doubles(const std::string& s, double* out, int n) {
  const char* b = s.data();
  const char* e = b + s.size();
  for (int k = 0; k < n; k++) {
    while (b < e && (*b == ' ' || *b == '\t' || *b == '\n' || *b == '\r' || *b == ',')) b++;
    if (*b == '+') b++;
    auto r = std::from_chars(b, e, out[k]);
    if (r.ec != std::errc()) throw std::runtime_error("URDF: cannot parse number list '" + s + "'");
    b = r.ptr;
  }
}
double parse_double(const std::string& s) {
  double v;
  parse_doubles(s, &v, 1);
  return v;
}

void mat_mul(const double* A, const double* B, double* C) {
  double T[9];
  for (int i = 0; i < 3; i++)
    for (int j = 0; j < 3; j++) T[i * 3 + j] = A[i * 3] * B[j] + A[i * 3 + 1] * B[3 + j] + A[i * 3 + 2] * B[6 + j];
  std::memcpy(C, T, sizeof T);
}
void mat_vec(const double* A, const double* x, double* y) {
  double t[3];
  for (int i = 0; i < 3; i++) t[i] = A[i * 3] * x[0] + A[i * 3 + 1] * x[1] + A[i * 3 + 2] * x[2];
  std::memcpy(y, t, sizeof t);
}
Placement compose(const Placement& a, const Placement& b) {
  Placement c;
  mat_mul(a.R, b.R, c.R);
  mat_vec(a.R, b.p, c.p);
  for (int k = 0; k < 3; k++) c.p[k] += a.p[k];
  return c;
}
Placement identity() {
  Placement P;
  const double I[9] = {1, 0, 0, 0, 1, 0, 0, 0, 1};
  std::memcpy(P.R, I, sizeof I);
  P.p[0] = P.p[1] = P.p[2] = 0;
  return P;
}
void rpy_to_R(const double rpy[3], double* R) {
  double phi = rpy[0] / 2, the = rpy[1] / 2, psi = rpy[2] / 2;
  double x = std::sin(phi) * std::cos(the) * std::cos(psi) - std::cos(phi) * std::sin(the) * std::sin(psi);
  double y = std::cos(phi) * std::sin(the) * std::cos(psi) + std::sin(phi) * std::cos(the) * std::sin(psi);
  double z = std::cos(phi) * std::cos(the) * std::sin(psi) - std::sin(phi) * std::sin(the) * std::cos(psi);
  double w = std::cos(phi) * std::cos(the) * std::cos(psi) + std::sin(phi) * std::sin(the) * std::sin(psi);
  double n = std::sqrt(x * x + y * y + z * z + w * w);
  x /= n; y /= n; z /= n; w /= n;
  R[0] = 1 - 2 * (y * y + z * z); R[1] = 2 * (x * y - w * z);     R[2] = 2 * (x * z + w * y);
  R[3] = 2 * (x * y + w * z);     R[4] = 1 - 2 * (x * x + z * z); R[5] = 2 * (y * z - w * x);
  R[6] = 2 * (x * z - w * y);     R[7] = 2 * (y * z + w * x);     R[8] = 1 - 2 * (x * x + y * y);
}
Placement origin_of(const XmlNode* elem) {
  Placement P = identity();
  if (!elem) return P;
  const XmlNode* o = elem->child("origin");
  if (!o) return P;
  double xyz[3] = {0, 0, 0}, rpy[3] = {0, 0, 0};
  if (auto* a = o->attr("xyz")) parse_doubles(*a, xyz, 3);
  if (auto* a = o->attr("rpy")) parse_doubles(*a, rpy, 3);
  rpy_to_R(rpy, P.R);
  std::memcpy(P.p, xyz, sizeof xyz);
  return P;
}

// Link inertial (m, com c, Ic about com, in link frame) -> origin form in link frame.
BodyInertia link_inertia(const XmlNode* link) {
  BodyInertia B;
  const XmlNode* in = link->child("inertial");
  if (!in) return B;
  Placement o = origin_of(in);
  double m = 0;
  if (auto* me = in->child("mass"))
    if (auto* v = me->attr("value")) m = parse_double(*v);
  double Iu[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
  if (auto* ie = in->child("inertia")) {
    auto get = [&](const char* k) { auto* a = ie->attr(k); return a ? parse_double(*a) : 0.0; };
    double xx = get("ixx"), xy = get("ixy"), xz = get("ixz"), yy = get("iyy"), yz = get("iyz"), zz = get("izz");
    double t[9] = {xx, xy, xz, xy, yy, yz, xz, yz, zz};
    std::memcpy(Iu, t, sizeof t);
  }
  double Ic[9], T[9], Rt[9];
  for (int i = 0; i < 3; i++)
    for (int j = 0; j < 3; j++) Rt[i * 3 + j] = o.R[j * 3 + i];
  mat_mul(o.R, Iu, T);
  mat_mul(T, Rt, Ic);
  const double* c = o.p;
  double cc = c[0] * c[0] + c[1] * c[1] + c[2] * c[2];
  B.m = m;
  for (int k = 0; k < 3; k++) B.h[k] = m * c[k];
  // I = Ic + m (|c|^2 I - c c^T)
  B.I[0] = Ic[0] + m * (cc - c[0] * c[0]);
  B.I[1] = Ic[1] - m * c[0] * c[1];
  B.I[2] = Ic[2] - m * c[0] * c[2];
  B.I[3] = Ic[4] + m * (cc - c[1] * c[1]);
  B.I[4] = Ic[5] - m * c[1] * c[2];
  B.I[5] = Ic[8] + m * (cc - c[2] * c[2]);
  return B;
}

// Express an origin-form inertia given in frame B in frame A (x_A = R x_B + p).
BodyInertia transport(const BodyInertia& B, const Placement& P) {
  BodyInertia O;
  O.m = B.m;
  double hr[3];
  mat_vec(P.R, B.h, hr);
  for (int k = 0; k < 3; k++) O.h[k] = hr[k] + B.m * P.p[k];
  double I9[9] = {B.I[0], B.I[1], B.I[2], B.I[1], B.I[3], B.I[4], B.I[2], B.I[4], B.I[5]};
  double T[9], Rt[9], Ir[9];
  for (int i = 0; i < 3; i++)
    for (int j = 0; j < 3; j++) Rt[i * 3 + j] = P.R[j * 3 + i];
  mat_mul(P.R, I9, T);
  mat_mul(T, Rt, Ir);
  // I_A = R I_B R^T + m(|p|^2 I - p p^T) + 2 (hr.p) I - p hr^T - hr p^T
  const double* p = P.p;
  double pp = p[0] * p[0] + p[1] * p[1] + p[2] * p[2];
  double hp = hr[0] * p[0] + hr[1] * p[1] + hr[2] * p[2];
  auto at = [&](int i, int j) {
    double d = (i == j) ? (B.m * pp + 2 * hp) : 0.0;
    return Ir[i * 3 + j] + d - B.m * p[i] * p[j] - p[i] * hr[j] - hr[i] * p[j];
  };
  O.I[0] = at(0, 0); O.I[1] = at(0, 1); O.I[2] = at(0, 2);
  O.I[3] = at(1, 1); O.I[4] = at(1, 2); O.I[5] = at(2, 2);
  return O;
}
void add_inertia(BodyInertia& A, const BodyInertia& B) {
  A.m += B.m;
  for (int k = 0; k < 3; k++) A.h[k] += B.h[k];
  for (int k = 0; k < 6; k++) A.I[k] += B.I[k];
}

bool is_identity(const double* R) {
  return R[0] == 1 && R[4] == 1 && R[8] == 1 && R[1] == 0 && R[2] == 0 && R[3] == 0 && R[5] == 0 && R[6] == 0 &&
         R[7] == 0;
}

// Rotation C (row-major) with C e_z = a for a unit axis a. Coordinate axes get exact
// integer rotations; other axes the orthonormal basis of Duff et al., "Building an
// Orthonormal Basis, Revisited" (JCGT 2017), with a as the third column.
void rotation_to_axis(const double a[3], double C[9]) {
  const double ex[9] = {0, 0, 1, 0, 1, 0, -1, 0, 0}, nex[9] = {0, 0, -1, 0, 1, 0, 1, 0, 0};
  const double ey[9] = {1, 0, 0, 0, 0, 1, 0, -1, 0}, ney[9] = {1, 0, 0, 0, 0, -1, 0, 1, 0};
  const double ez[9] = {1, 0, 0, 0, 1, 0, 0, 0, 1}, nez[9] = {1, 0, 0, 0, -1, 0, 0, 0, -1};
  const double* exact = nullptr;
  if (a[1] == 0 && a[2] == 0) exact = a[0] > 0 ? ex : nex;
  else if (a[0] == 0 && a[2] == 0) exact = a[1] > 0 ? ey : ney;
  else if (a[0] == 0 && a[1] == 0) exact = a[2] > 0 ? ez : nez;
  if (exact) {
    std::memcpy(C, exact, 9 * sizeof(double));
    return;
  }
  const double sg = std::copysign(1.0, a[2]);
  const double k = -1.0 / (sg + a[2]);
  const double b = a[0] * a[1] * k;
  const double b1[3] = {1.0 + sg * a[0] * a[0] * k, sg * b, -sg * a[0]};
  const double b2[3] = {b, sg + a[1] * a[1] * k, -a[1]};
  for (int r = 0; r < 3; r++) {
    C[r * 3 + 0] = b1[r];
    C[r * 3 + 1] = b2[r];
    C[r * 3 + 2] = a[r];
  }
}

// out = A^T B (3x3 row-major)
void mat_tmul(const double* A, const double* B, double* out) {
  for (int i = 0; i < 3; i++)
    for (int j = 0; j < 3; j++) out[i * 3 + j] = A[0 * 3 + i] * B[0 * 3 + j] + A[1 * 3 + i] * B[1 * 3 + j] + A[2 * 3 + i] * B[2 * 3 + j];
}
// out = A^T x
void mat_tvec(const double* A, const double* x, double* out) {
  for (int i = 0; i < 3; i++) out[i] = A[0 * 3 + i] * x[0] + A[1 * 3 + i] * x[1] + A[2 * 3 + i] * x[2];
}

}  // namespace

// Builds the depth-first tree from link inertias (origin form, link frame) and joint
// descriptions keyed by name (std::map: byte-wise name order for siblings).
Model* Model::build_tree(const std::map<std::string, BodyInertia>& links, const std::map<std::string, JointSpec>& jdesc,
                         const double g[3]) {
  std::map<std::string, std::string> parent_joint_of;  // child link -> joint name
  for (auto& kv : jdesc) {
    const JointSpec& d = kv.second;
    if (!links.count(d.parent) || !links.count(d.child))
      throw std::runtime_error("URDF: joint " + kv.first + " references an unknown link");
    if (parent_joint_of.count(d.child)) throw std::runtime_error("URDF: link " + d.child + " has two parents");
    parent_joint_of[d.child] = kv.first;
  }
  std::vector<std::string> roots;
  for (auto& kv : links)
    if (!parent_joint_of.count(kv.first)) roots.push_back(kv.first);
  if (roots.size() != 1) throw std::runtime_error("URDF: expected exactly one root link");
  std::map<std::string, std::vector<std::string>> children;  // link -> joint names (sorted)
  for (auto& kv : jdesc) children[kv.second.parent].push_back(kv.first);

  auto* M = new Model;
  std::memcpy(M->gravity, g, sizeof(double) * 3);
  HostJoint uni;
  uni.name = "universe";
  uni.placement = identity();
  M->joints.push_back(uni);
  M->joints[0].inertia = links.at(roots[0]);
  M->bodies.push_back({roots[0], 0, identity()});
  std::function<void(const std::string&, int)> visit = [&](const std::string& link, int body_idx) {
    const HostBody pb = M->bodies[body_idx];
    for (auto& jn : children[link]) {
      const JointSpec& d = jdesc.at(jn);
      Placement P = compose(pb.placement, d.origin);
      BodyInertia Yc = links.at(d.child);
      if (d.type == "fixed") {
        add_inertia(M->joints[pb.joint].inertia, transport(Yc, P));
        M->bodies.push_back({d.child, pb.joint, P});
      } else {
        HostJoint J;
        J.name = jn;
        J.parent = pb.joint;
        J.placement = P;
        J.inertia = Yc;
        J.lower = d.lower;
        J.upper = d.upper;
        if (d.type == "revolute") J.kind = JK_REVOLUTE;
        else if (d.type == "continuous") J.kind = JK_CONTINUOUS;
        else if (d.type == "prismatic") J.kind = JK_PRISMATIC;
        else if (d.type == "floating") J.kind = JK_FREEFLYER;
        else throw std::runtime_error("URDF: unsupported joint type '" + d.type + "' (joint " + jn + ")");
        if (J.kind != JK_FREEFLYER) {
          double n = std::sqrt(d.axis[0] * d.axis[0] + d.axis[1] * d.axis[1] + d.axis[2] * d.axis[2]);
          if (!(n > 0)) throw std::runtime_error("URDF: zero joint axis (joint " + jn + ")");
          for (int k = 0; k < 3; k++) J.axis[k] = d.axis[k] / n;
        }
        J.depth = M->joints[pb.joint].depth + 1;
        M->joints.push_back(J);
        M->bodies.push_back({d.child, int(M->joints.size()) - 1, identity()});
      }
      visit(d.child, int(M->bodies.size()) - 1);
    }
  };
  visit(roots[0], 0);
  int nq = 0, nv = 0;
  for (auto& J : M->joints) {
    int jq = 0, jv = 0;
    switch (J.kind) {
      case JK_REVOLUTE: case JK_PRISMATIC: jq = 1; jv = 1; break;
      case JK_CONTINUOUS: jq = 2; jv = 1; break;
      case JK_FREEFLYER: jq = 7; jv = 6; break;
      default: break;
    }
    J.idx_q = nq; J.idx_v = nv; J.nq = jq; J.nv = jv;
    nq += jq; nv += jv;
  }
  M->nq_int_ = nq;
  M->nv_ = nv;
  // default orders: tree order for joints, URDF tree order for links
  std::vector<std::string> jn, ln;
  for (size_t j = 1; j < M->joints.size(); j++) jn.push_back(M->joints[j].name);
  for (auto& b : M->bodies) ln.push_back(b.name);
  M->set_joint_order(jn);
  M->set_link_order(ln);
  return M;
}

Model* Model::from_urdf(const std::string& xml, const double g[3]) {
  auto root = parse_xml(xml);
  if (root->name != "robot") throw std::runtime_error("URDF: root element is not <robot>");
  std::map<std::string, BodyInertia> links;
  std::map<std::string, JointSpec> jdesc;
  for (auto& c : root->children) {
    if (c->name == "link") {
      auto* n = c->attr("name");
      if (!n) throw std::runtime_error("URDF: link without name");
      if (links.count(*n)) throw std::runtime_error("URDF: duplicate link " + *n);
      links[*n] = link_inertia(c.get());
    } else if (c->name == "joint") {
      auto* n = c->attr("name");
      auto* t = c->attr("type");
      if (!n || !t) throw std::runtime_error("URDF: joint without name or type");
      const XmlNode* pe = c->child("parent");
      const XmlNode* ce = c->child("child");
      if (!pe || !ce || !pe->attr("link") || !ce->attr("link"))
        throw std::runtime_error("URDF: joint " + *n + " lacks parent/child");
      JointSpec d;
      d.type = *t;
      d.parent = *pe->attr("link");
      d.child = *ce->attr("link");
      d.origin = origin_of(c.get());
      d.axis[0] = 1; d.axis[1] = 0; d.axis[2] = 0;
      if (auto* ax = c->child("axis"))
        if (auto* a = ax->attr("xyz")) parse_doubles(*a, d.axis, 3);
      if (auto* lim = c->child("limit")) {
        if (auto* lo = lim->attr("lower")) parse_doubles(*lo, &d.lower, 1);
        if (auto* up = lim->attr("upper")) parse_doubles(*up, &d.upper, 1);
      }
      if (jdesc.count(*n)) throw std::runtime_error("URDF: duplicate joint " + *n);
      jdesc[*n] = d;
    }
  }
  return build_tree(links, jdesc, g);
}

namespace {
Placement pose7(const double* p) {
  Placement P;
  const double w = p[3], x = p[4], y = p[5], z = p[6];
  P.R[0] = 1 - 2 * (y * y + z * z); P.R[1] = 2 * (x * y - w * z);     P.R[2] = 2 * (x * z + w * y);
  P.R[3] = 2 * (x * y + w * z);     P.R[4] = 1 - 2 * (x * x + z * z); P.R[5] = 2 * (y * z - w * x);
  P.R[6] = 2 * (x * z - w * y);     P.R[7] = 2 * (y * z + w * x);     P.R[8] = 1 - 2 * (x * x + y * y);
  P.p[0] = p[0]; P.p[1] = p[1]; P.p[2] = p[2];
  return P;
}
Placement inverse(const Placement& a) {
  Placement b;
  for (int i = 0; i < 3; i++)
    for (int j = 0; j < 3; j++) b.R[i * 3 + j] = a.R[j * 3 + i];
  double t[3];
  mat_vec(b.R, a.p, t);
  for (int k = 0; k < 3; k++) b.p[k] = -t[k];
  return b;
}
}  // namespace

// Restates python/py_package/wrapper/urdf_exporter.py:21-152 (export_link, export_joint,
// export_kinematic_chain_urdf with force_fix_root) and create_pinocchio_model
// (python/py_package/wrapper/pinocchio_model.py:317-326) without the XML round trip.
Model* Model::from_articulation(const ArtLink* links, int nlinks, const ArtJoint* joints, int njoints,
                                const double g[3], bool force_fix_root) {
  if (nlinks <= 0) throw std::runtime_error("articulation without links");
  std::map<std::string, BodyInertia> L;
  std::map<std::string, JointSpec> J;
  L["world"] = BodyInertia();
  for (int i = 0; i < nlinks; i++) {
    // inertial: origin = c.o.m. pose, diagonal principal inertia in that frame
    const Placement o = pose7(links[i].cmass_pose);
    double Ic[9], T[9], Rt[9];
    const double Id[9] = {links[i].inertia[0], 0, 0, 0, links[i].inertia[1], 0, 0, 0, links[i].inertia[2]};
    for (int r = 0; r < 3; r++)
      for (int c = 0; c < 3; c++) Rt[r * 3 + c] = o.R[c * 3 + r];
    mat_mul(o.R, Id, T);
    mat_mul(T, Rt, Ic);
    BodyInertia B;
    const double m = links[i].mass, *c = o.p;
    const double cc = c[0] * c[0] + c[1] * c[1] + c[2] * c[2];
    B.m = m;
    for (int k = 0; k < 3; k++) B.h[k] = m * c[k];
    B.I[0] = Ic[0] + m * (cc - c[0] * c[0]);
    B.I[1] = Ic[1] - m * c[0] * c[1];
    B.I[2] = Ic[2] - m * c[0] * c[2];
    B.I[3] = Ic[4] + m * (cc - c[1] * c[1]);
    B.I[4] = Ic[5] - m * c[1] * c[2];
    B.I[5] = Ic[8] + m * (cc - c[2] * c[2]);
    L["link_" + std::to_string(i)] = B;
  }
  std::vector<std::string> active;
  for (int k = 0; k < njoints; k++) {
    const ArtJoint& a = joints[k];
    if (a.child < 0 || a.child >= nlinks || a.parent >= nlinks)
      throw std::runtime_error("articulation joint references an unknown link");
    const std::string ci = std::to_string(a.child), name = "joint_" + ci;
    JointSpec js;
    js.axis[0] = 1; js.axis[1] = 0; js.axis[2] = 0;
    if (a.parent < 0) {
      js.type = (a.type == ART_FIXED || force_fix_root) ? "fixed" : "floating";
      js.parent = "world";
      js.child = "link_" + ci;
      js.origin = identity();
      J[name] = js;
      if (js.type != "fixed") active.push_back(name);
      continue;
    }
    switch (a.type) {
      case ART_FIXED: js.type = "fixed"; break;
      case ART_PRISMATIC: js.type = "prismatic"; break;
      case ART_REVOLUTE: js.type = (a.lower < -1e5 && a.upper > 1e5) ? "continuous" : "revolute"; break;
      default: throw std::runtime_error("invalid joint type for a non-root joint");
    }
    js.parent = "link_" + std::to_string(a.parent);
    js.child = "link_dummy_" + ci;
    js.origin = pose7(a.pose_in_parent);
    js.lower = a.lower;
    js.upper = a.upper;
    J[name] = js;
    JointSpec dj;
    dj.type = "fixed";
    dj.parent = "link_dummy_" + ci;
    dj.child = "link_" + ci;
    dj.origin = inverse(pose7(a.pose_in_child));
    dj.axis[0] = 0; dj.axis[1] = 0; dj.axis[2] = 0;
    J["joint_dummy_" + ci] = dj;
    L["link_dummy_" + ci] = BodyInertia();
    if (js.type != "fixed") active.push_back(name);
  }
  Model* M = build_tree(L, J, g);
  try {
    std::vector<std::string> lo;
    for (int i = 0; i < nlinks; i++) lo.push_back("link_" + std::to_string(i));
    M->set_joint_order(active);
    M->set_link_order(lo);
  } catch (...) {
    delete M;
    throw;
  }
  return M;
}

void Model::set_joint_order(const std::vector<std::string>& names) {
  std::vector<int> ids;
  std::set<int> seen;
  for (auto& n : names) {
    int id = -1;
    for (size_t j = 1; j < joints.size(); j++)
      if (joints[j].name == n) id = int(j);
    if (id < 0 || seen.count(id)) throw InvalidArgument("invalid names in setJointOrder");
    seen.insert(id);
    ids.push_back(id);
  }
  int count = 0;
  for (int id : ids) count += joints[id].nv;
  if (count != nv_) throw std::runtime_error("setJointOrder failed");
  std::vector<int> qc(joints.size(), -1), vc(joints.size(), -1);
  int qo = 0, vo = 0;
  for (int id : ids) {
    qc[id] = qo;
    vc[id] = vo;
    qo += joints[id].kind == JK_FREEFLYER ? 7 : 1;
    vo += joints[id].nv;
  }
  std::lock_guard<std::mutex> lk(mu_);
  qcol_ = qc;
  vcol_ = vc;
  nq_ext_ = qo;
  rebuild_table();
}

void Model::set_link_order(const std::vector<std::string>& names) {
  std::vector<int> lb;
  for (auto& n : names) {
    int id = -1;
    for (size_t b = 0; b < bodies.size(); b++)
      if (bodies[b].name == n) id = int(b);
    if (id < 0) throw InvalidArgument("invalid names in setLinkOrder");
    lb.push_back(id);
  }
  std::lock_guard<std::mutex> lk(mu_);
  link_bodies_ = lb;
  rebuild_table();
}

int Model::max_depth() const {
  int d = 0;
  for (auto& J : joints) d = std::max(d, J.depth);
  return d;
}
bool Model::has_free_flyer() const {
  for (auto& J : joints)
    if (J.kind == JK_FREEFLYER) return true;
  return false;
}

uint64_t Model::next_uid() {
  static std::atomic<uint64_t> counter{1};
  return counter++;
}

void Model::rebuild_table() {
  version_++;
  int nj = njoints(), nl = int(link_bodies_.size());
  table_.assign(model_table_bytes(nj, nl), 0);
  auto* hdr = reinterpret_cast<DModel*>(table_.data());
  hdr->nj = nj;
  hdr->nv = nv_;
  hdr->nq_ext = nq_ext_;
  hdr->nlinks = nl;
  hdr->max_depth = max_depth();
  int nff = 0;
  for (auto& J : joints) nff += J.kind == JK_FREEFLYER;
  hdr->n_free_flyer = nff;
  std::memcpy(hdr->gravity, gravity, sizeof(double) * 3);
  auto* dj = const_cast<DJoint*>(model_joints(hdr));
  auto* df = const_cast<DFrame*>(model_frames(hdr));
  // Canonical frames: C_j with C_j e_z = axis_j for 1-DoF joints. A joint keeps its own
  // frame (C_j = 1, general axis) when its placement, seen from its parent's table frame,
  // and some link frame on it are both unrotated: there the axis products cost less than
  // the rotation C_j would add to that link's pose. Parents come first in depth-first order.
  std::vector<char> canon(nj, 0), bare_link(nj, 0);
  for (int l = 0; l < nl; l++) {
    const HostBody& B = bodies[link_bodies_[l]];
    if (is_identity(B.placement.R)) bare_link[B.joint] = 1;
  }
  const double I3[9] = {1, 0, 0, 0, 1, 0, 0, 0, 1};
  std::memcpy(df[0].C, I3, sizeof I3);
  for (int j = 1; j < nj; j++) {
    const HostJoint& J = joints[j];
    const bool axial = J.kind == JK_REVOLUTE || J.kind == JK_CONTINUOUS || J.kind == JK_PRISMATIC;
    double Reff[9];
    mat_tmul(df[J.parent].C, J.placement.R, Reff);
    canon[j] = axial && !(is_identity(Reff) && bare_link[j]);
    if (canon[j]) rotation_to_axis(J.axis, df[j].C);
    else std::memcpy(df[j].C, I3, sizeof I3);
  }
  for (int j = 0; j < nj; j++) {
    const HostJoint& J = joints[j];
    DJoint& D = dj[j];
    const double* Cj = df[j].C;
    const double* Cp = df[j > 0 ? J.parent : 0].C;
    // placement in canonical frames: R' = Cp^T R Cj, p' = Cp^T p
    double T[9];
    mat_tmul(Cp, J.placement.R, T);
    mat_mul(T, Cj, D.R);
    mat_tvec(Cp, J.placement.p, D.p);
    if (canon[j]) {
      D.axis[0] = 0;
      D.axis[1] = 0;
      D.axis[2] = 1.0;
    } else {
      std::memcpy(D.axis, J.axis, sizeof D.axis);
    }
    // body inertia in the canonical frame: h' = Cj^T h, I' = Cj^T I Cj
    D.m = J.inertia.m;
    mat_tvec(Cj, J.inertia.h, D.h);
    const double* I = J.inertia.I;
    const double Im[9] = {I[0], I[1], I[2], I[1], I[3], I[4], I[2], I[4], I[5]};
    double Ir[9];
    mat_tmul(Cj, Im, T);
    mat_mul(T, Cj, Ir);
    D.I[0] = Ir[0];
    D.I[1] = 0.5 * (Ir[1] + Ir[3]);
    D.I[2] = 0.5 * (Ir[2] + Ir[6]);
    D.I[3] = Ir[4];
    D.I[4] = 0.5 * (Ir[5] + Ir[7]);
    D.I[5] = Ir[8];
    D.parent = J.parent;
    D.kind = J.kind;
    D.axis_kind = canon[j] ? AX_Z : AX_GENERAL;
    D.flags = is_identity(D.R) ? JF_ROT_IDENTITY : 0;
    D.qcol = j < int(qcol_.size()) ? qcol_[j] : -1;
    D.vcol = j < int(vcol_.size()) ? vcol_[j] : -1;
    D.nv = J.nv;
    D.depth = J.depth;
    D.ivx = J.idx_v;
    D.subtree_end = j + 1;
  }
  // subtrees are contiguous in depth-first order: extend each parent's end to its children's
  for (int j = nj - 1; j >= 1; j--)
    if (dj[j].parent > 0 && dj[dj[j].parent].subtree_end < dj[j].subtree_end)
      dj[dj[j].parent].subtree_end = dj[j].subtree_end;
  auto* dl = const_cast<DLink*>(model_links(hdr));
  for (int l = 0; l < nl; l++) {
    const HostBody& B = bodies[link_bodies_[l]];
    // link frame relative to its joint's canonical frame: Cj^T (R, p)
    const double* Cj = df[B.joint].C;
    mat_tmul(Cj, B.placement.R, dl[l].R);
    mat_tvec(Cj, B.placement.p, dl[l].p);
    dl[l].joint = B.joint;
    dl[l].flags = is_identity(dl[l].R) ? JF_ROT_IDENTITY : 0;
  }
  // device copies are stale now
  for (auto& kv : dev_) {
    int cur;
    if (cudaGetDevice(&cur) == cudaSuccess) {
      cudaSetDevice(kv.first);
      cudaFree(kv.second);
      cudaSetDevice(cur);
    }
  }
  dev_.clear();
  for (auto& kv : dev_team_) {
    int cur;
    if (cudaGetDevice(&cur) == cudaSuccess) {
      cudaSetDevice(kv.first.first);
      cudaFree(kv.second);
      cudaSetDevice(cur);
    }
  }
  dev_team_.clear();
  team_cp_.clear();
}

const DModel* Model::device_table(int* err) {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) {
    *err = 1;
    return nullptr;
  }
  std::lock_guard<std::mutex> lk(mu_);
  auto it = dev_.find(dev);
  if (it != dev_.end()) return static_cast<const DModel*>(it->second);
  void* p = nullptr;
  if (cudaMalloc(&p, table_.size()) != cudaSuccess) {
    *err = 2;
    return nullptr;
  }
  if (cudaMemcpy(p, table_.data(), table_.size(), cudaMemcpyHostToDevice) != cudaSuccess) {
    cudaFree(p);
    *err = 3;
    return nullptr;
  }
  dev_[dev] = p;
  return static_cast<const DModel*>(p);
}

// Team table for L lanes per environment (layout in step_kernel.cuh). The trunk starts
// empty with the root subtrees as branches; the heaviest branch's root is moved into the
// trunk (its children become branches) while that lowers trunk cost + the heaviest lane's
// cost, lanes being filled longest-branch-first. Joint cost: 1, a free flyer 4.
std::vector<int> Model::team_table(int L, int* critical_path) const {
  const auto* hdr = reinterpret_cast<const DModel*>(table_.data());
  const DJoint* J = model_joints(hdr);
  const int nj = hdr->nj;
  std::vector<std::vector<int>> kids(nj);
  for (int j = 1; j < nj; j++) kids[J[j].parent].push_back(j);
  std::vector<int> cost(nj, 0), sub(nj, 0);
  for (int j = 1; j < nj; j++) cost[j] = J[j].nv == 6 ? 4 : 1;
  for (int j = nj - 1; j >= 1; j--) {
    sub[j] += cost[j];
    if (J[j].parent > 0) sub[J[j].parent] += sub[j];
  }
  std::vector<int> trunk, branches = kids[0];
  int trunk_cost = 0;
  int best = 1 << 30;
  std::vector<int> best_trunk, best_owner;
  for (;;) {
    std::vector<int> order = branches;
    std::stable_sort(order.begin(), order.end(), [&](int x, int y) { return sub[x] > sub[y]; });
    std::vector<int> load(L, 0), role_of(nj, -1);
    for (int r : order) {
      const int lane = int(std::min_element(load.begin(), load.end()) - load.begin());
      load[lane] += sub[r];
      role_of[r] = lane;
    }
    const int cp = trunk_cost + *std::max_element(load.begin(), load.end());
    if (cp < best) {
      best = cp;
      best_trunk = trunk;
      best_owner.assign(nj, -1);
      for (int j = 1; j < nj; j++) {  // a branch joint belongs to its branch root's lane
        int r = j;
        while (r > 0 && role_of[r] < 0 && std::find(trunk.begin(), trunk.end(), r) == trunk.end()) r = J[r].parent;
        if (r > 0 && role_of[r] >= 0) best_owner[j] = role_of[r];
      }
    }
    if (branches.empty()) break;
    const int h = *std::max_element(branches.begin(), branches.end(), [&](int x, int y) { return sub[x] < sub[y]; });
    if (kids[h].empty()) break;
    branches.erase(std::find(branches.begin(), branches.end(), h));
    trunk.push_back(h);
    trunk_cost += cost[h];
    for (int c : kids[h]) branches.push_back(c);
  }
  std::sort(best_trunk.begin(), best_trunk.end());
  std::vector<std::vector<int>> lanes(L);
  for (int j = 1; j < nj; j++)
    if (best_owner[j] >= 0) lanes[best_owner[j]].push_back(j);
  size_t smax = 0;
  for (auto& l : lanes) smax = std::max(smax, l.size());
  std::vector<int> attach;
  for (int t : best_trunk)
    for (int c : kids[t])
      if (best_owner[c] >= 0) {
        attach.push_back(t);
        break;
      }
  if (critical_path) *critical_path = best;
  std::vector<int> tab = {L, int(best_trunk.size()), int(smax), int(attach.size())};
  tab.insert(tab.end(), best_trunk.begin(), best_trunk.end());
  for (auto& l : lanes) {
    tab.insert(tab.end(), l.begin(), l.end());
    tab.insert(tab.end(), smax - l.size(), 0);
  }
  tab.insert(tab.end(), attach.begin(), attach.end());
  tab.insert(tab.end(), best_owner.begin(), best_owner.end());
  return tab;
}


int Model::team_critical_path(int L) {
  std::lock_guard<std::mutex> lk(mu_);
  auto it = team_cp_.find(L);
  if (it != team_cp_.end()) return it->second;
  int cp = 0;
  team_table(L, &cp);
  team_cp_[L] = cp;
  return cp;
}

const int* Model::device_team(int L, int* err) {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) {
    *err = 1;
    return nullptr;
  }
  std::lock_guard<std::mutex> lk(mu_);
  auto key = std::make_pair(dev, L);
  auto it = dev_team_.find(key);
  if (it != dev_team_.end()) return static_cast<const int*>(it->second);
  const std::vector<int> t = team_table(L);
  void* p = nullptr;
  if (cudaMalloc(&p, sizeof(int) * t.size()) != cudaSuccess) {
    *err = 2;
    return nullptr;
  }
  if (cudaMemcpy(p, t.data(), sizeof(int) * t.size(), cudaMemcpyHostToDevice) != cudaSuccess) {
    cudaFree(p);
    *err = 3;
    return nullptr;
  }
  dev_team_[key] = p;
  return static_cast<const int*>(p);
}

const DModel* Model::find_device_table() {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return nullptr;
  std::lock_guard<std::mutex> lk(mu_);
  auto it = dev_.find(dev);
  return it == dev_.end() ? nullptr : static_cast<const DModel*>(it->second);
}

Model::~Model() {
  for (auto& kv : dev_) {
    int cur;
    if (cudaGetDevice(&cur) == cudaSuccess) {
      cudaSetDevice(kv.first);
      cudaFree(kv.second);
      cudaSetDevice(cur);
    }
  }
  for (auto& kv : dev_team_) {
    int cur;
    if (cudaGetDevice(&cur) == cudaSuccess) {
      cudaSetDevice(kv.first.first);
      cudaFree(kv.second);
      cudaSetDevice(cur);
    }
  }
}

void Model::random_configuration(int64_t n, uint64_t seed, double* q) const {
  for (int j = 1; j < njoints(); j++) {
    const HostJoint& J = joints[j];
    if (J.kind == JK_FREEFLYER)
      throw std::runtime_error("random configuration: free-flyer joint " + J.name + " has no position limits");
    if ((J.kind == JK_REVOLUTE || J.kind == JK_PRISMATIC) && !(J.lower <= J.upper))
      throw std::runtime_error("random configuration: joint " + J.name + " has lower limit above upper limit");
  }
  std::mt19937_64 rng(seed);
  const double pi = 3.14159265358979323846;
  for (int64_t e = 0; e < n; e++)
    for (int j = 1; j < njoints(); j++) {
      const HostJoint& J = joints[j];
      const double u = double(rng() >> 11) * (1.0 / 9007199254740992.0);  // [0, 1), 53 bits
      double& x = q[e * nq_ext_ + qcol_[j]];
      if (J.kind == JK_CONTINUOUS) x = -pi + 2 * pi * u;
      else x = J.lower + (J.upper - J.lower) * u;
    }
}

}  // namespace sgdyn
