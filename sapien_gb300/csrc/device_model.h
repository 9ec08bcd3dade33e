// Flat, depth-first joint table read by the kernels. One contiguous buffer:
//   DModel header | DJoint[nj] (joint 0 = universe, unused) | DLink[nlinks] | DFrame[nj]
// Every environment of a batch reads the same table, so all lanes of a warp load the
// same address (a broadcast through L1).
//
// Canonical joint frames. Each revolute / continuous / prismatic joint's frame is rotated
// by a constant C (DFrame) so that its axis is +z: the model's joint frame F and the
// table's frame F' = F C. Placements, axes, body inertias and link offsets are stored in
// the F' frames, so a joint rotation is Rz(q) and a motion subspace is a column of the
// world rotation (no axis products). World-frame results and link frames are unchanged;
// only a quantity reported in a joint frame (the CLIK error) is rotated back by C.
#pragma once
#ifdef __CUDACC_RTC__
// run-time compilation: no standard headers
typedef long long int64_t;
typedef unsigned long size_t;
#else
#include <cstddef>
#include <cstdint>
#endif

#ifdef __CUDACC__
#define SG_HD __host__ __device__ __forceinline__
#else
#define SG_HD inline
#endif

namespace sgdyn {

enum JointKind : int { JK_NONE = 0, JK_REVOLUTE = 1, JK_PRISMATIC = 2, JK_CONTINUOUS = 3, JK_FREEFLYER = 4 };
enum AxisKind : int { AX_X = 0, AX_Y = 1, AX_Z = 2, AX_GENERAL = 3 };
enum JointFlags : int { JF_ROT_IDENTITY = 1 };

struct alignas(16) DJoint {
  double R[9];   // placement rotation (parent joint frame <- this joint frame at q = 0), row-major
  double p[3];   // placement translation
  double axis[3];  // +z for revolute / continuous / prismatic (canonical frame), else 0
  double m;      // body inertia carried by this joint, about the joint origin:
  double h[3];   //   first moment m*c
  double I[6];   //   rotational inertia about the origin: xx xy xz yy yz zz
  int parent;    // parent joint (0 = universe)
  int kind;      // JointKind
  int axis_kind; // AxisKind
  int flags;     // JointFlags
  int qcol;      // external q column of the first coordinate
  int vcol;      // external v column of the first velocity
  int nv;        // 1, or 6 for a free flyer
  int depth;     // 1 for children of the universe
  int ivx;       // first velocity index in depth-first (tree) order
  int subtree_end;  // one past the last joint of this joint's subtree (depth-first order)
  int pad_[4];
};
static_assert(sizeof(DJoint) == 256, "DJoint layout");

struct alignas(16) DLink {
  double R[9];  // link frame in its joint frame
  double p[3];
  int joint;
  int flags;    // JF_ROT_IDENTITY when the placement rotation is exactly identity
  int pad_[2];
};
static_assert(sizeof(DLink) == 112, "DLink layout");

struct alignas(16) DFrame {
  double C[9];  // model joint frame <- table joint frame, row-major (identity for free flyers)
  double pad_;
};
static_assert(sizeof(DFrame) == 80, "DFrame layout");

struct alignas(16) DModel {
  int nj;       // joints incl. universe
  int nv;
  int nq_ext;
  int nlinks;
  int max_depth;
  int n_free_flyer;
  int pad_[2];
  double gravity[3];
  double pad2_;
};
static_assert(sizeof(DModel) == 64, "DModel layout");

SG_HD const DJoint* model_joints(const DModel* m) {
  return reinterpret_cast<const DJoint*>(reinterpret_cast<const char*>(m) + sizeof(DModel));
}
SG_HD const DLink* model_links(const DModel* m) {
  return reinterpret_cast<const DLink*>(reinterpret_cast<const char*>(m) + sizeof(DModel) +
                                        sizeof(DJoint) * size_t(m->nj));
}
SG_HD const DFrame* model_frames(const DModel* m) {
  return reinterpret_cast<const DFrame*>(reinterpret_cast<const char*>(model_links(m)) +
                                         sizeof(DLink) * size_t(m->nlinks));
}
SG_HD size_t model_table_bytes(int nj, int nlinks) {
  return sizeof(DModel) + sizeof(DJoint) * size_t(nj) + sizeof(DLink) * size_t(nlinks) +
         sizeof(DFrame) * size_t(nj);
}

}  // namespace sgdyn
