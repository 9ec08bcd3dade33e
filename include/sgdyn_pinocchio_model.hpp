/* C++ drop-in for sapien::PinocchioModel (pinocchio/pinocchio_model.h:27-130) over the C ABI
 * of sgdyn.h. Header only; link with -lsgdyn.
 *
 * Method names, argument order and defaults follow the reference class. The reference
 * takes and returns Eigen types; this header has no Eigen dependency, so vectors are
 * std::vector<double> and matrices a row-major sgdyn::Matrix. The single-configuration
 * methods run the library's sweeps compiled for the host (sgdyn_host_*), on the calling
 * thread, as the reference computes on the CPU; handle() gives the model for the batched
 * device entry points of sgdyn.h. Errors follow the reference's split: bad joint or link
 * names throw std::invalid_argument, everything else std::runtime_error (with the library's
 * message). Like the reference object it is not thread-safe (it caches the last forward
 * kinematics and Jacobian configuration) and not copyable.
 */
#ifndef SGDYN_PINOCCHIO_MODEL_HPP
#define SGDYN_PINOCCHIO_MODEL_HPP

#include <cstdint>
#include <memory>
#include <random>
#include <stdexcept>
#include <string>
#include <tuple>
#include <vector>

#include "sgdyn.h"

namespace sgdyn {

/* Row-major dense matrix. */
struct Matrix {
  int rows = 0, cols = 0;
  std::vector<double> data;
  Matrix() = default;
  Matrix(int r, int c) : rows(r), cols(c), data(size_t(r) * size_t(c), 0.0) {}
  double& operator()(int r, int c) { return data[size_t(r) * cols + c]; }
  double operator()(int r, int c) const { return data[size_t(r) * cols + c]; }
};

/* A rigid transform as sapien::Pose: float position and unit quaternion (w, x, y, z). */
struct Pose {
  float p[3] = {0, 0, 0};
  float q[4] = {1, 0, 0, 0};
};

class PinocchioModel {
 public:
  /* fromURDFXML (pinocchio_model.cpp:39-47). */
  static std::unique_ptr<PinocchioModel> fromURDFXML(const std::string& urdf, const double gravity[3]) {
    sgdyn_model* m = nullptr;
    check(sgdyn_model_from_urdf(urdf.c_str(), gravity, &m));
    return std::unique_ptr<PinocchioModel>(new PinocchioModel(m));
  }
  ~PinocchioModel() { sgdyn_model_free(m_); }
  PinocchioModel(const PinocchioModel&) = delete;
  PinocchioModel& operator=(const PinocchioModel&) = delete;

  /* setJointOrder / setLinkOrder (pinocchio_model.cpp:99-140). */
  void setJointOrder(const std::vector<std::string>& names) {
    std::vector<const char*> c;
    for (auto& s : names) c.push_back(s.c_str());
    check(sgdyn_model_set_joint_order(m_, c.data(), int(c.size())));
    joint_order_set_ = true;
    refresh();
  }
  void setLinkOrder(const std::vector<std::string>& names) {
    std::vector<const char*> c;
    for (auto& s : names) c.push_back(s.c_str());
    check(sgdyn_model_set_link_order(m_, c.data(), int(c.size())));
    link_order_set_ = true;
    fk_.clear();
    refresh();
  }

  /* getRandomConfiguration (pinocchio_model.cpp:142-144): nv x 1. */
  Matrix getRandomConfiguration() {
    std::random_device rd;
    const uint64_t seed = (uint64_t(rd()) << 32) ^ uint64_t(rd());
    Matrix out(nq_, 1);
    check(sgdyn_model_random_configuration(m_, 1, seed, out.data.data()));
    return out;
  }

  /* computeForwardKinematics + getLinkPose (pinocchio_model.cpp:146-161). */
  void computeForwardKinematics(const std::vector<double>& qpos) {
    requireOrder(qpos);
    fk_.assign(size_t(nlinks_) * 7, 0.0);
    check(sgdyn_host_step(m_, 1, SGDYN_OP_FK, qpos.data(), nullptr, nullptr, nullptr, fk_.data(),
                          nullptr, nullptr, nullptr, nullptr, SGDYN_ENV_MAJOR, 1));
  }
  Pose getLinkPose(uint32_t index) const {
    checkLink(index);
    if (fk_.empty()) throw std::runtime_error("computeForwardKinematics must be called before getLinkPose");
    Pose p;
    for (int k = 0; k < 3; k++) p.p[k] = float(fk_[size_t(index) * 7 + k]);
    for (int k = 0; k < 4; k++) p.q[k] = float(fk_[size_t(index) * 7 + 3 + k]);
    return p;
  }

  /* computeFullJacobian + getLinkJacobian (pinocchio_model.cpp:163-186): 6 x nv, WORLD, or
   * the link frame with local = true. */
  void computeFullJacobian(const std::vector<double>& qpos) {
    requireOrder(qpos);
    jac_q_ = qpos;
  }
  Matrix getLinkJacobian(uint32_t index, bool local = false) const {
    checkLink(index);
    if (jac_q_.empty()) throw std::runtime_error("computeFullJacobian must be called before getLinkJacobian");
    Matrix J(6, nv_);
    check(sgdyn_host_compute_link_jacobian(m_, 1, int(index), local ? 1 : 0, jac_q_.data(), J.data.data(),
                                           SGDYN_ENV_MAJOR, 1));
    return J;
  }
  /* computeSingleLinkLocalJacobian (pinocchio_model.cpp:188-199). */
  Matrix computeSingleLinkLocalJacobian(const std::vector<double>& qpos, uint32_t index) const {
    requireOrder(qpos);
    checkLink(index);
    Matrix J(6, nv_);
    check(sgdyn_host_compute_link_jacobian(m_, 1, int(index), 1, qpos.data(), J.data.data(), SGDYN_ENV_MAJOR, 1));
    return J;
  }

  /* computeGeneralizedMassMatrix (pinocchio_model.cpp:201-206). */
  Matrix computeGeneralizedMassMatrix(const std::vector<double>& qpos) const {
    requireOrder(qpos);
    Matrix M(nv_, nv_);
    check(sgdyn_host_step(m_, 1, SGDYN_OP_MASS_MATRIX, qpos.data(), nullptr, nullptr, nullptr, nullptr, nullptr,
                          M.data.data(), nullptr, nullptr, SGDYN_ENV_MAJOR, 1));
    return M;
  }
  /* computeCoriolisMatrix (pinocchio_model.cpp:208-212). */
  Matrix computeCoriolisMatrix(const std::vector<double>& qpos, const std::vector<double>& qvel) const {
    requireOrder(qpos);
    requireSize(qvel, nv_, "qvel");
    Matrix C(nv_, nv_);
    check(sgdyn_host_compute_coriolis_matrix(m_, 1, qpos.data(), qvel.data(), C.data.data(), SGDYN_ENV_MAJOR, 1));
    return C;
  }
  /* computeInverseDynamics (pinocchio_model.cpp:214-219). */
  std::vector<double> computeInverseDynamics(const std::vector<double>& qpos, const std::vector<double>& qvel,
                                             const std::vector<double>& qacc) const {
    requireOrder(qpos);
    requireSize(qvel, nv_, "qvel");
    requireSize(qacc, nv_, "qacc");
    std::vector<double> tau(static_cast<size_t>(nv_));
    check(sgdyn_host_step(m_, 1, SGDYN_OP_INVERSE_DYNAMICS, qpos.data(), qvel.data(), qacc.data(), nullptr, nullptr,
                          nullptr, nullptr, tau.data(), nullptr, SGDYN_ENV_MAJOR, 1));
    return tau;
  }
  /* computeForwardDynamics (pinocchio_model.cpp:221-226). */
  std::vector<double> computeForwardDynamics(const std::vector<double>& qpos, const std::vector<double>& qvel,
                                             const std::vector<double>& qf) const {
    requireOrder(qpos);
    requireSize(qvel, nv_, "qvel");
    requireSize(qf, nv_, "qf");
    std::vector<double> qacc(static_cast<size_t>(nv_));
    check(sgdyn_host_step(m_, 1, SGDYN_OP_FORWARD_DYNAMICS, qpos.data(), qvel.data(), nullptr, qf.data(), nullptr,
                          nullptr, nullptr, nullptr, qacc.data(), SGDYN_ENV_MAJOR, 1));
    return qacc;
  }

  /* computeInverseKinematics (pinocchio_model.cpp:228-300): (q, success, error); an empty
   * initialQpos starts from the neutral configuration, an empty activeQmask frees every
   * joint. */
  std::tuple<std::vector<double>, bool, std::vector<double>> computeInverseKinematics(
      uint32_t linkIdx, const Pose& pose, const std::vector<double>& initialQpos = {},
      const std::vector<int>& activeQmask = {}, double eps = 1e-4, int maxIter = 1000, double dt = 1e-1,
      double damp = 1e-6) const {
    checkLink(linkIdx);
    if (!joint_order_set_ && nv_ > 0) throw std::runtime_error("posS2P failed");
    if (!initialQpos.empty()) requireOrder(initialQpos);
    if (!activeQmask.empty() && int(activeQmask.size()) != nv_)
      throw std::runtime_error("activeQmask must have one entry per degree of freedom");
    const double target[7] = {pose.p[0], pose.p[1], pose.p[2], pose.q[0], pose.q[1], pose.q[2], pose.q[3]};
    std::vector<double> q(static_cast<size_t>(nq_)), err(6);
    int success = 0;
    check(sgdyn_host_compute_inverse_kinematics(m_, 1, int(linkIdx), target,
                                                initialQpos.empty() ? nullptr : initialQpos.data(),
                                                activeQmask.empty() ? nullptr : activeQmask.data(), eps, maxIter, dt,
                                                damp, q.data(), &success, err.data(), SGDYN_ENV_MAJOR, 1));
    return std::make_tuple(q, success != 0, err);
  }

  /* The library's model, for the batched device entry points of sgdyn.h. */
  sgdyn_model* handle() const { return m_; }
  int dof() const { return nv_; }

 private:
  explicit PinocchioModel(sgdyn_model* m) : m_(m) { refresh(); }

  static void check(int rc) {
    if (rc == SGDYN_OK) return;
    if (rc == SGDYN_ERR_INVALID_ARGUMENT) throw std::invalid_argument(sgdyn_last_error());
    throw std::runtime_error(sgdyn_last_error());
  }
  void refresh() {
    int nq = 0, nv = 0, nl = 0, nj = 0;
    check(sgdyn_model_info(m_, &nq, &nv, &nl, &nj));
    nq_ = nq;
    nv_ = nv;
    nlinks_ = link_order_set_ ? nl : 0;
  }
  void requireOrder(const std::vector<double>& qpos) const {
    if ((!joint_order_set_ && nv_ > 0) || int(qpos.size()) != nq_) throw std::runtime_error("posS2P failed");
  }
  static void requireSize(const std::vector<double>& v, int n, const char* what) {
    if (int(v.size()) != n) throw std::runtime_error(std::string(what) + " has the wrong size");
  }
  void checkLink(uint32_t index) const {
    if (int64_t(index) >= int64_t(nlinks_)) throw std::runtime_error("link index out of bound");
  }

  sgdyn_model* m_ = nullptr;
  bool joint_order_set_ = false, link_order_set_ = false;
  int nq_ = 0, nv_ = 0, nlinks_ = 0;
  std::vector<double> fk_, jac_q_;
};

}  // namespace sgdyn

#endif /* SGDYN_PINOCCHIO_MODEL_HPP */
