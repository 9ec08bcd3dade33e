// Exercises include/sgdyn_pinocchio_model.hpp as a C++ caller of sapien::PinocchioModel
// would. Reads from stdin: the URDF path, the joint names, the link names, the end-effector
// link index, then q, qd, qdd, tau and an IK start configuration (one line each); prints
// every result as "name v0 v1 ..." lines for the test to compare with the oracle.
#include <cstdio>
#include <iostream>
#include <sstream>
#include <string>
#include <vector>

#include "sgdyn_pinocchio_model.hpp"

static std::vector<std::string> words(const std::string& line) {
  std::istringstream s(line);
  std::vector<std::string> out;
  for (std::string w; s >> w;) out.push_back(w);
  return out;
}
static std::vector<double> numbers(const std::string& line) {
  std::istringstream s(line);
  std::vector<double> out;
  for (double x; s >> x;) out.push_back(x);
  return out;
}
static void put(const char* name, const std::vector<double>& v) {
  std::printf("%s", name);
  for (double x : v) std::printf(" %.17g", x);
  std::printf("\n");
}

int main() {
  std::string path, jl, ll, eel, ql, qdl, qddl, taul, q0l;
  std::getline(std::cin, path);
  std::getline(std::cin, jl);
  std::getline(std::cin, ll);
  std::getline(std::cin, eel);
  std::getline(std::cin, ql);
  std::getline(std::cin, qdl);
  std::getline(std::cin, qddl);
  std::getline(std::cin, taul);
  std::getline(std::cin, q0l);
  std::string urdf;
  {
    FILE* f = std::fopen(path.c_str(), "rb");
    if (!f) return 2;
    char buf[4096];
    for (size_t n; (n = std::fread(buf, 1, sizeof buf, f)) > 0;) urdf.append(buf, n);
    std::fclose(f);
  }
  const double g[3] = {0, 0, -9.81};
  auto model = sgdyn::PinocchioModel::fromURDFXML(urdf, g);
  // a joint order before any call: computing without one fails as posS2P does
  try {
    model->computeGeneralizedMassMatrix(numbers(ql));
    std::printf("error_before_order none\n");
  } catch (const std::runtime_error& e) {
    std::printf("error_before_order runtime_error\n");
  }
  try {
    model->setJointOrder({"no_such_joint"});
    std::printf("error_bad_name none\n");
  } catch (const std::invalid_argument&) {
    std::printf("error_bad_name invalid_argument\n");
  }
  model->setJointOrder(words(jl));
  const auto links = words(ll);
  model->setLinkOrder(links);
  const uint32_t ee = uint32_t(std::stoul(eel));
  const auto q = numbers(ql), qd = numbers(qdl), qdd = numbers(qddl), tau = numbers(taul), q0 = numbers(q0l);
  model->computeForwardKinematics(q);
  std::vector<double> poses;
  for (uint32_t l = 0; l < links.size(); l++) {
    const sgdyn::Pose p = model->getLinkPose(l);
    for (float x : p.p) poses.push_back(x);
    for (float x : p.q) poses.push_back(x);
  }
  put("poses", poses);
  try {
    model->getLinkPose(uint32_t(links.size()));
    std::printf("error_bad_link none\n");
  } catch (const std::runtime_error&) {
    std::printf("error_bad_link runtime_error\n");
  }
  model->computeFullJacobian(q);
  put("jacobian_world", model->getLinkJacobian(ee).data);
  put("jacobian_local", model->getLinkJacobian(ee, true).data);
  put("jacobian_single", model->computeSingleLinkLocalJacobian(q, ee).data);
  put("mass_matrix", model->computeGeneralizedMassMatrix(q).data);
  put("coriolis", model->computeCoriolisMatrix(q, qd).data);
  put("inverse_dynamics", model->computeInverseDynamics(q, qd, qdd));
  put("forward_dynamics", model->computeForwardDynamics(q, qd, tau));
  // IK towards the end-effector pose at q from q0, fixed iteration count (eps = 0)
  const sgdyn::Pose target = model->getLinkPose(ee);
  auto ik = model->computeInverseKinematics(ee, target, q0, {}, 0.0, 50, 0.3, 1e-3);
  put("ik_q", std::get<0>(ik));
  put("ik_err", std::get<2>(ik));
  std::printf("ik_success %d\n", std::get<1>(ik) ? 1 : 0);
  put("random_configuration", model->getRandomConfiguration().data);
  return 0;
}
