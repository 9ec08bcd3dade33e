// Host-side kinematic model: URDF -> depth-first joint tree with Pinocchio's
// conventions, the SAPIEN<->tree joint permutation, link frames, and the flat
// device tables the kernels read.
#pragma once
#include <cstdint>
#include <map>
#include <mutex>
#include <string>
#include <vector>

#include "device_model.h"

namespace sgdyn {

struct Placement {
  double R[9];  // row-major rotation, parent <- child
  double p[3];
};

struct BodyInertia {  // about the frame origin: h = m c, I = Ic + m [c]x^T [c]x
  double m = 0;
  double h[3] = {0, 0, 0};
  double I[6] = {0, 0, 0, 0, 0, 0};  // xx xy xz yy yz zz
};

struct HostJoint {
  std::string name;
  int parent = 0;
  int kind = 0;  // JK_*
  double axis[3] = {0, 0, 0};
  Placement placement;
  BodyInertia inertia;
  int idx_q = 0, idx_v = 0, nq = 0, nv = 0, depth = 0;
  double lower = 0, upper = 0;  // position limits of a revolute or prismatic joint
};

struct JointSpec {  // a URDF joint before tree building
  std::string type, parent, child;
  Placement origin;
  double axis[3];
  double lower = 0, upper = 0;  // <limit lower upper>, 0 when absent as in URDF
};

// An articulation as SAPIEN describes it (PhysxArticulationLinkComponent / Joint getters):
// poses are (x y z qw qx qy qz); inertia are principal moments in the c.o.m. frame.
struct ArtLink {
  double mass;
  double cmass_pose[7];
  double inertia[3];
};
enum ArtJointType : int { ART_FIXED = 0, ART_REVOLUTE = 1, ART_PRISMATIC = 2, ART_FREE = 3 };
struct ArtJoint {
  int type;    // ArtJointType
  int parent;  // parent link index, -1 for the root joint
  int child;   // child link index
  double pose_in_parent[7];
  double pose_in_child[7];
  double lower, upper;  // limits of the joint's single coordinate
};

struct HostBody {  // a BODY frame (one per URDF link)
  std::string name;
  int joint;
  Placement placement;
};

class Model {
 public:
  // Builds from URDF XML; the root link is welded to the universe (joint 0).
  static Model* from_urdf(const std::string& xml, const double gravity[3]);
  // Builds the tree SAPIEN's URDF exporter would describe for this articulation
  // (link_{i} / joint_{child} names, a dummy link per moving joint, joint axis x), then
  // sets the joint order to the active joints in articulation order and the link order to
  // the articulation's links, as create_pinocchio_model does.
  static Model* from_articulation(const ArtLink* links, int nlinks, const ArtJoint* joints, int njoints,
                                  const double gravity[3], bool force_fix_root);
  // Builds from link inertias (origin form, in the link frame) and joint descriptions,
  // both keyed by name; the root link is welded to the universe.
  static Model* build_tree(const std::map<std::string, BodyInertia>& links,
                           const std::map<std::string, JointSpec>& joints, const double gravity[3]);

  void set_joint_order(const std::vector<std::string>& names);
  void set_link_order(const std::vector<std::string>& names);

  // getRandomConfiguration (pinocchio_model.cpp:142-144): n rows of external q, each
  // revolute or prismatic coordinate uniform in its [lower, upper], each continuous angle
  // uniform in [-pi, pi); std::mt19937_64 seeded with `seed`, 53-bit uniforms, so the
  // samples are the same on every platform. Throws for a free flyer (no position limits).
  void random_configuration(int64_t n, uint64_t seed, double* q) const;

  int njoints() const { return int(joints.size()); }
  int nq_ext() const { return nq_ext_; }
  int nv() const { return nv_; }
  int nq_int() const { return nq_int_; }
  int nlinks() const { return int(link_bodies_.size()); }
  int max_depth() const;
  bool has_free_flyer() const;

  // Device table for the current CUDA device (uploaded on first use).
  const DModel* device_table(int* err);
  // Device table for the current CUDA device if it was already uploaded, else null;
  // never allocates.
  const DModel* find_device_table();
  // Host copy of the packed table (for tests and for the heterogeneous packer).
  const std::vector<unsigned char>& host_table() const { return table_; }

  // Team table for L lanes per environment (layout in step_kernel.cuh: TeamLanes);
  // *critical_path receives the joint-cost length of the trunk + heaviest lane.
  std::vector<int> team_table(int L, int* critical_path = nullptr) const;
  // Its device copy on the current device (uploaded on first use), or null.
  const int* device_team(int L, int* err);
  // The critical path of team_table(L), cached.
  int team_critical_path(int L);
  // Lanes per environment for the single-model entry points: 0 = automatic, 1, 2, 4, 8.
  int lanes = 0;

  std::vector<HostJoint> joints;  // [0] = universe
  std::vector<HostBody> bodies;
  double gravity[3] = {0, 0, -9.81};
  int ext_qcol_of_joint(int j) const { return qcol_[j]; }
  int ext_vcol_of_joint(int j) const { return vcol_[j]; }
  int link_body(int link) const { return link_bodies_[link]; }

  ~Model();

  // Identity of this model and of the current contents of its tables (bumped whenever
  // the tables are rebuilt), for caches keyed on the table contents.
  uint64_t uid() const { return uid_; }
  uint64_t table_version() const { return version_; }

 private:
  void rebuild_table();
  int nq_ext_ = 0, nv_ = 0, nq_int_ = 0;
  std::vector<int> qcol_, vcol_;   // per joint: external q / v column of its first coordinate
  std::vector<int> link_bodies_;   // external link index -> bodies[]
  std::vector<unsigned char> table_;
  std::map<int, void*> dev_;       // device ordinal -> device copy of table_
  std::map<std::pair<int, int>, void*> dev_team_;  // (device, L) -> device team table
  std::map<int, int> team_cp_;                       // L -> critical path
  std::mutex mu_;
  uint64_t uid_ = next_uid();
  uint64_t version_ = 0;
  static uint64_t next_uid();
};

}  // namespace sgdyn
