// Run-time specialisation of the fused sweep (NVRTC).
//
// For a given model and op set the generated translation unit holds the model's kernel
// tables as compile-time constants and instantiates step_env_t with StaticTab, so every
// joint loop unrolls into straight-line code with constant parents, axes, placements and
// inertias: no dynamic local-memory indexing, no branches on joint kind, and one large
// basic block in which the scheduler can fill the FP64 pipe's issue shadow. The arithmetic
// is the same sequence of operations as the generic kernel (results are bitwise equal).
//
// libnvrtc and the driver library are opened with dlopen on first use, so the package
// loads on machines without them; compiled cubins are cached in memory per (source,
// device) and on disk under $SGDYN_JIT_CACHE (default ~/.cache/sapien_gb300/jit).
#include "jit.h"

#include <cuda.h>
#include <dlfcn.h>
#include <nvrtc.h>
#include <sys/stat.h>
#include <unistd.h>

#include <atomic>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <map>
#include <tuple>
#include <mutex>
#include <sstream>
#include <vector>

#include "model.h"

namespace sgdyn {

extern const char* const kJitHeaderNames[];
extern const char* const kJitHeaderSources[];
extern const int kJitHeaderCount;

namespace {

struct Api {
  bool loaded = false;
  std::string why;
  decltype(&nvrtcCreateProgram) createProgram = nullptr;
  decltype(&nvrtcCompileProgram) compileProgram = nullptr;
  decltype(&nvrtcGetCUBINSize) getCUBINSize = nullptr;
  decltype(&nvrtcGetCUBIN) getCUBIN = nullptr;
  decltype(&nvrtcGetProgramLogSize) getLogSize = nullptr;
  decltype(&nvrtcGetProgramLog) getLog = nullptr;
  decltype(&nvrtcDestroyProgram) destroyProgram = nullptr;
  decltype(&nvrtcVersion) version = nullptr;
  decltype(&cuModuleLoadData) moduleLoadData = nullptr;
  decltype(&cuModuleGetFunction) moduleGetFunction = nullptr;
  decltype(&cuLaunchKernel) launchKernel = nullptr;
};

Api load_api() {
  Api a;
  void* nv = dlopen("libnvrtc.so.13", RTLD_NOW | RTLD_LOCAL);
  if (!nv) nv = dlopen("libnvrtc.so", RTLD_NOW | RTLD_LOCAL);
  void* cu = dlopen("libcuda.so.1", RTLD_NOW | RTLD_LOCAL);
  if (!nv || !cu) {
    a.why = !nv ? "libnvrtc not found" : "libcuda.so.1 not found";
    return a;
  }
#define SG_SYM(lib, field, name)                                  \
  a.field = reinterpret_cast<decltype(a.field)>(dlsym(lib, name)); \
  if (!a.field) {                                                 \
    a.why = std::string("missing symbol ") + name;                \
    return a;                                                     \
  }
  SG_SYM(nv, createProgram, "nvrtcCreateProgram")
  SG_SYM(nv, compileProgram, "nvrtcCompileProgram")
  SG_SYM(nv, getCUBINSize, "nvrtcGetCUBINSize")
  SG_SYM(nv, getCUBIN, "nvrtcGetCUBIN")
  SG_SYM(nv, getLogSize, "nvrtcGetProgramLogSize")
  SG_SYM(nv, getLog, "nvrtcGetProgramLog")
  SG_SYM(nv, destroyProgram, "nvrtcDestroyProgram")
  SG_SYM(nv, version, "nvrtcVersion")
  SG_SYM(cu, moduleLoadData, "cuModuleLoadData")
  SG_SYM(cu, moduleGetFunction, "cuModuleGetFunction")
  SG_SYM(cu, launchKernel, "cuLaunchKernel")
#undef SG_SYM
  a.loaded = true;
  return a;
}

Api& api() {
  static Api a = load_api();
  return a;
}

std::mutex g_mu;
int g_enable = -1;  // -1: read SGDYN_JIT on first use
int64_t g_min_n = 2048;
// Trees above this many joints (incl. the universe) keep the generic kernels: fully
// unrolled sweeps of large trees overflow the instruction cache and spill, and ran slower.
int g_max_joints = 16;
std::map<std::string, CUfunction> g_functions;  // key: source hash + device
std::map<std::string, std::string> g_failed;    // key -> reason
// fast path: (model uid, table version, ops, device) -> kernel, so a launch does no string work
std::map<std::tuple<uint64_t, uint64_t, int, int, int>, CUfunction> g_by_model;
std::map<std::tuple<uint64_t, uint64_t, int, int, int>, std::string> g_failed_by_model;

void read_env_config() {
  if (g_enable >= 0) return;
  const char* e = std::getenv("SGDYN_JIT");
  g_enable = (e && std::strcmp(e, "0") == 0) ? 0 : 1;
  if (const char* m = std::getenv("SGDYN_JIT_MIN_N")) g_min_n = std::atoll(m);
  if (const char* m = std::getenv("SGDYN_JIT_MAX_JOINTS")) g_max_joints = std::atoi(m);
}

const char* const kNvrtcOptions[] = {"--gpu-architecture=sm_103a", "-std=c++17", "-lineinfo"};
constexpr int kNvrtcOptionCount = 3;

uint64_t fnv1a(const std::string& s) {
  uint64_t h = 1469598103934665603ull;
  for (unsigned char c : s) {
    h ^= c;
    h *= 1099511628211ull;
  }
  return h;
}

std::string num(double x) {
  char b[40];
  std::snprintf(b, sizeof b, "%.17g", x);
  return b;
}

template <class It>
std::string list(It b, It e) {
  std::string s;
  for (It i = b; i != e; ++i) s += (i == b ? "" : ", ") + num(*i);
  return s;
}

// The rollout's backward kernels stay generic: specialised, they came out slower (the
// fully unrolled reverse sweep spills heavily).
enum JitKind {
  JIT_STEP = 0, JIT_ROLLOUT_FWD = 1, JIT_RNEA_VJP = 2, JIT_ABA_VJP = 3, JIT_ROLLOUT_FWD3 = 4, JIT_ROLLOUT_REV3 = 5,
  JIT_ABA3 = 6, JIT_STEP_ROLES = 7
};
const char* kernel_name(int kind) {
  static const char* const names[] = {"sgjit_step",    "sgjit_rollout_forward",  "sgjit_rnea_vjp",
                                      "sgjit_aba_vjp", "sgjit_rollout_forward3", "sgjit_rollout_reverse3",
                                      "sgjit_aba3",    "sgjit_step_roles"};
  return names[kind];
}
bool team3_kind(int kind) { return kind == JIT_ROLLOUT_FWD3 || kind == JIT_ROLLOUT_REV3 || kind == JIT_ABA3; }
// Environments per block of each kernel kind (blocks of 32 threads, but JIT_STEP_ROLES: one
// warp per role of the team, 32 environments).
int envs_per_block(int kind) { return team3_kind(kind) ? 10 : 32; }
// The role-warp sweep's key packs the lanes per environment above the op bits.
constexpr int kRoleLanesShift = 8;

// Columns of the largest tree a model may have (63 moving joints, one of them a free flyer).
constexpr int kMaxTreeColumns = 63 + 5;

// Tree columns of the joint table: ancestors of each column, nearest first (empty if the
// numbering does not put parents first), and external column numbers.
struct Columns {
  std::vector<std::vector<int>> anc;
  std::vector<int> ext;
  bool ok = true;
};
Columns tree_columns(const DJoint* J, int nj, int nv) {
  Columns C;
  C.anc.resize(size_t(nv));
  C.ext.assign(size_t(nv), 0);
  std::vector<int> par(size_t(nv), -1);
  for (int i = 1; i < nj; i++)
    for (int k = 0; k < J[i].nv; k++) {
      const int a = J[i].ivx + k;
      C.ext[a] = J[i].vcol + k;
      par[a] = k > 0 ? a - 1 : (J[i].parent > 0 ? J[J[i].parent].ivx + J[J[i].parent].nv - 1 : -1);
      if (par[a] >= a) C.ok = false;
    }
  if (C.ok)
    for (int a = 0; a < nv; a++)
      for (int c = par[a]; c >= 0; c = par[c]) C.anc[a].push_back(c);
  return C;
}

// The mass-matrix route of forward dynamics as straight-line code for one tree (the steps of
// FdLoops in step_kernel.cuh with every index a constant, so that M lives in registers).
void emit_fd(std::ostringstream& o, const Columns& C, int nv) {
  auto at = [](int a, int b) { return a * (a + 1) / 2 + b; };
  const char* head = "  template <class Tab";
  o << "struct kFd {\n";
  o << head << ">\n  static __device__ __forceinline__ void fill(const Tab&, double* H, const sgdyn::Mot* S, "
       "const sgdyn::Mot* F) {\n";
  for (int a = 0; a < nv; a++) {
    o << "    H[" << at(a, a) << "] = sgdyn::dot6(S[" << a << "], F[" << a << "]);\n";
    for (int c : C.anc[a]) o << "    H[" << at(a, c) << "] = sgdyn::dot6(S[" << c << "], F[" << a << "]);\n";
  }
  o << "  }\n";
  o << head << ", class St>\n  static __device__ __forceinline__ void store_M(const Tab&, const double* H, const St& st) "
       "{\n";
  for (int a = 0; a < nv; a++)
    for (int b = 0; b < nv; b++) {
      int idx = -1;
      if (a == b) idx = at(a, a);
      for (int c : C.anc[a])
        if (c == b) idx = at(a, b);
      for (int c : C.anc[b])
        if (c == a) idx = at(b, a);
      o << "    st(" << C.ext[a] << ", " << C.ext[b] << ", " << (idx >= 0 ? "H[" + std::to_string(idx) + "]" : "0.0")
        << ");\n";
    }
  o << "  }\n";
  o << head << ">\n  static __device__ __forceinline__ void matvec_add(const Tab&, const double* H, const double* x, "
       "double* y) {\n";
  for (int a = 0; a < nv; a++) {
    o << "    y[" << a << "] = fma(H[" << at(a, a) << "], x[" << a << "], y[" << a << "]);\n";
    for (int c : C.anc[a]) {
      o << "    y[" << a << "] = fma(H[" << at(a, c) << "], x[" << c << "], y[" << a << "]);\n";
      o << "    y[" << c << "] = fma(H[" << at(a, c) << "], x[" << a << "], y[" << c << "]);\n";
    }
  }
  o << "  }\n";
  o << head << ">\n  static __device__ __forceinline__ void factor(const Tab&, double* H, double* D) {\n";
  for (int a = nv - 1; a >= 0; a--) {
    o << "    { const double r = 1.0 / H[" << at(a, a) << "]; D[" << a << "] = r;\n";
    for (size_t t = 0; t < C.anc[a].size(); t++) {
      const int c = C.anc[a][t];
      o << "      { const double f = H[" << at(a, c) << "] * r;\n";
      o << "        H[" << at(c, c) << "] = fma(-f, H[" << at(a, c) << "], H[" << at(c, c) << "]);\n";
      for (int d : C.anc[c])
        o << "        H[" << at(c, d) << "] = fma(-f, H[" << at(a, d) << "], H[" << at(c, d) << "]);\n";
      o << "        H[" << at(a, c) << "] = f; }\n";
    }
    o << "    }\n";
  }
  o << "  }\n";
  o << head << ">\n  static __device__ __forceinline__ void solve(const Tab&, const double* H, const double* D, "
       "double* x) {\n";
  for (int a = nv - 1; a >= 0; a--)
    for (int c : C.anc[a])
      o << "    x[" << c << "] = fma(-H[" << at(a, c) << "], x[" << a << "], x[" << c << "]);\n";
  for (int a = 0; a < nv; a++) {
    o << "    x[" << a << "] *= D[" << a << "];\n";
    for (int c : C.anc[a]) o << "    x[" << a << "] = fma(-H[" << at(a, c) << "], x[" << c << "], x[" << a << "]);\n";
  }
  o << "  }\n};\n";
}

std::string generate_source(const Model& M, int kind, int ops) {
  const auto& t = M.host_table();
  const auto* hdr = reinterpret_cast<const DModel*>(t.data());
  const DJoint* J = model_joints(hdr);
  const DLink* L = model_links(hdr);
  const int nj = hdr->nj, nl = hdr->nlinks;
  std::ostringstream o;
  if (kind == JIT_STEP_ROLES) o << "#include \"se3.cuh\"\n";
  o << (kind == JIT_STEP || kind == JIT_STEP_ROLES ? "#include \"step_kernel.cuh\"\n"
        : team3_kind(kind) ? "#include \"team3.cuh\"\n"
                           : "#include \"diff_kernels.cuh\"\n");
  o << "namespace sgjit {\n";
  o << "__device__ constexpr sgdyn::DModel kM = {" << hdr->nj << ", " << hdr->nv << ", " << hdr->nq_ext << ", "
    << hdr->nlinks << ", " << hdr->max_depth << ", " << hdr->n_free_flyer << ", {0, 0}, {"
    << list(hdr->gravity, hdr->gravity + 3) << "}, 0.0};\n";
  o << "__device__ constexpr sgdyn::DJoint kJT[" << nj << "] = {\n";
  for (int j = 0; j < nj; j++) {
    const DJoint& d = J[j];
    o << " {{" << list(d.R, d.R + 9) << "}, {" << list(d.p, d.p + 3) << "}, {" << list(d.axis, d.axis + 3) << "}, "
      << num(d.m) << ", {" << list(d.h, d.h + 3) << "}, {" << list(d.I, d.I + 6) << "}, " << d.parent << ", " << d.kind
      << ", " << d.axis_kind << ", " << d.flags << ", " << d.qcol << ", " << d.vcol << ", " << d.nv << ", " << d.depth
      << ", " << d.ivx << ", " << d.subtree_end << ", {0, 0, 0, 0}},\n";
  }
  o << "};\n";
  o << "__device__ constexpr sgdyn::DLink kLT[" << (nl > 0 ? nl : 1) << "] = {\n";
  for (int l = 0; l < nl; l++)
    o << " {{" << list(L[l].R, L[l].R + 9) << "}, {" << list(L[l].p, L[l].p + 3) << "}, " << L[l].joint << ", "
      << L[l].flags << ", {0, 0}},\n";
  if (nl == 0) o << " {{1,0,0,0,1,0,0,0,1}, {0,0,0}, 0, 1, {0, 0}},\n";
  o << "};\n";
  const bool fd = kind == JIT_STEP && (ops & OP_FD_CRBA);
  if (fd) emit_fd(o, tree_columns(J, nj, hdr->nv), hdr->nv);
  o << "}  // namespace sgjit\n";
  int lanes = 0;
  if (kind == JIT_STEP_ROLES) {  // the team table as constants (roles are the block's warps)
    lanes = ops >> kRoleLanesShift;
    ops &= (1 << kRoleLanesShift) - 1;
    const std::vector<int> tt = M.team_table(lanes);
    o << "namespace sgjit {\n__device__ constexpr int kTT[" << tt.size() << "] = {";
    for (size_t k = 0; k < tt.size(); k++) o << (k ? ", " : "") << tt[k];
    o << "};\n}  // namespace sgjit\n";
  }
  const std::string tab = "sgdyn::StaticTab<" + std::to_string(nj) + ", " + std::to_string(hdr->nv) + ", " +
                          std::to_string(nl) + ", sgjit::kJT, sgjit::kLT, &sgjit::kM" + (fd ? ", sgjit::kFd" : "") +
                          ">()";
  if (kind == JIT_STEP_ROLES) {
    // rows: the environments' row indices (null: 0 .. count - 1); integrate != 0: then a
    // semi-implicit Euler step of q, qd (rows of a.q, a.qd, in place) from a.qdd_out
    o << "extern \"C\" __global__ void __launch_bounds__(" << 32 * lanes
      << ") sgjit_step_roles(const sgdyn::StepArgs a, const int* rows, long long count, double dt, int integrate) {\n"
      << "  __shared__ double xch[" << 32 * lanes << " * sgdyn::RoleTeam<0, sgjit::kTT>::kChunk];\n"
      << "  const int role = threadIdx.x >> 5, lane = threadIdx.x & 31;\n"
      << "  const long long i0 = (long long)blockIdx.x * 32 + lane;\n"
      << "  const bool valid = i0 < count;\n"
      << "  const long long i = valid ? i0 : count - 1;\n"
      << "  const long long e = rows ? (long long)rows[i] : i;\n"
      << "  switch (role) {\n";
    for (int r = 0; r < lanes; r++)
      o << "    case " << r << ": sgdyn::step_env_t<" << nj << ", " << ops << ">(" << tab << ", a, e, sgdyn::RoleTeam<" << r
        << ", sgjit::kTT>{xch, lane, valid}); break;\n";
    o << "  }\n"
      << "  if (integrate) {  // after every role has written its part of qdd\n"
      << "    __syncthreads();\n"
      << "    if (role == 0 && valid)\n"
      << "      sgdyn::integrate_env_t(" << tab << ", a.q.p + e * a.q.es, a.qd.p + e * a.qd.es, a.qdd_out.p + e * a.qdd_out.es, dt);\n"
      << "  }\n}\n";
    return o.str();
  }
  const char* args = (kind == JIT_STEP || kind == JIT_ABA3)                 ? "sgdyn::StepArgs"
                     : (kind == JIT_ROLLOUT_FWD || team3_kind(kind)) ? "sgdyn::RolloutArgs"
                                                                             : "sgdyn::VjpArgs";
  o << "extern \"C\" __global__ void __launch_bounds__(32) " << kernel_name(kind) << "(const " << args << " a) {\n";
  if (team3_kind(kind)) {  // ten environments per warp, three lanes each (team3.cuh)
    o << "  sgdyn::Team3 t = sgdyn::team3_of_lane(threadIdx.x);\n"
      << "  const long long e0 = (long long)blockIdx.x * 10 + t.base / 3;\n"
      << "  t.valid = t.valid && e0 < a.n;\n"
      << "  sgdyn::"
      << (kind == JIT_ROLLOUT_FWD3 ? "rollout_forward3_env" : kind == JIT_ABA3 ? "aba3_env" : "rollout_reverse3_env")
      << "<" << nj
      << ">(" << tab << ", t, a, e0 < a.n ? e0 : a.n - 1);\n}\n";
    return o.str();
  }
  o << "  const long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x;\n"
    << "  if (e >= a.n) return;\n";
  if (kind == JIT_STEP) o << "  sgdyn::step_env_t<" << nj << ", " << ops << ">(" << tab << ", a, e);\n}\n";
  else if (kind == JIT_ROLLOUT_FWD) o << "  sgdyn::rollout_forward_env<" << nj << ">(" << tab << ", a, e);\n}\n";
  else if (kind == JIT_RNEA_VJP) o << "  sgdyn::rnea_vjp_env<" << nj << ">(" << tab << ", a, e);\n}\n";
  else o << "  sgdyn::aba_vjp_env<" << nj << ">(" << tab << ", a, e);\n}\n";
  return o.str();
}

std::string cache_dir() {
  if (const char* d = std::getenv("SGDYN_JIT_CACHE")) return d;
  const char* home = std::getenv("HOME");
  return std::string(home ? home : "/tmp") + "/.cache/sapien_gb300/jit";
}

void mkdirs(const std::string& path) {
  std::string cur;
  for (size_t i = 0; i < path.size(); i++) {
    cur += path[i];
    if (path[i] == '/' && cur.size() > 1) mkdir(cur.c_str(), 0755);
  }
  mkdir(path.c_str(), 0755);
}

bool compile_cubin(const std::string& src, std::vector<char>* cubin, std::string* why) {
  Api& A = api();
  nvrtcProgram prog;
  if (A.createProgram(&prog, src.c_str(), "sgjit_kernel.cu", kJitHeaderCount, kJitHeaderSources, kJitHeaderNames) !=
      NVRTC_SUCCESS) {
    *why = "nvrtcCreateProgram failed";
    return false;
  }
  const char* const* opts = kNvrtcOptions;
  nvrtcResult rc = A.compileProgram(prog, kNvrtcOptionCount, opts);
  if (rc != NVRTC_SUCCESS) {
    size_t n = 0;
    A.getLogSize(prog, &n);
    std::string log(n, '\0');
    A.getLog(prog, &log[0]);
    *why = "nvrtc compile failed: " + log.substr(0, 2000);
    A.destroyProgram(&prog);
    return false;
  }
  size_t n = 0;
  A.getCUBINSize(prog, &n);
  cubin->resize(n);
  A.getCUBIN(prog, cubin->data());
  A.destroyProgram(&prog);
  return true;
}

CUfunction get_function_slow(const Model& M, int kind, int ops, int dev, std::string* why);

// Returns the specialised kernel for (M, kind, ops) on the current device, compiling if needed.
CUfunction get_function(const Model& M, int kind, int ops, std::string* why) {
  Api& A = api();
  if (!A.loaded) {
    *why = A.why;
    return nullptr;
  }
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) {
    *why = "no CUDA device";
    return nullptr;
  }
  const auto fast = std::make_tuple(M.uid(), M.table_version(), kind, ops, dev);
  auto it = g_by_model.find(fast);
  if (it != g_by_model.end()) return it->second;
  auto bad = g_failed_by_model.find(fast);
  if (bad != g_failed_by_model.end()) {
    *why = bad->second;
    return nullptr;
  }
  CUfunction fn = get_function_slow(M, kind, ops, dev, why);
  if (fn) g_by_model[fast] = fn;
  else g_failed_by_model[fast] = *why;
  return fn;
}

CUfunction get_function_slow(const Model& M, int kind, int ops, int dev, std::string* why) {
  Api& A = api();
  const std::string src = generate_source(M, kind, ops);
  int major = 0, minor = 0;
  A.version(&major, &minor);
  // The key covers the generated unit and the device headers it includes (so a rebuilt
  // library never picks up a cubin compiled from older headers) and the compiler version.
  static const uint64_t headers_hash = [] {
    std::string all;
    for (int k = 0; k < kNvrtcOptionCount; k++) all += std::string(kNvrtcOptions[k]) + '\n';
    for (int k = 0; k < kJitHeaderCount; k++) all += std::string(kJitHeaderNames[k]) + '\n' + kJitHeaderSources[k];
    return fnv1a(all);
  }();
  char hx[64];
  std::snprintf(hx, sizeof hx, "%016llx-%016llx-%d.%d", static_cast<unsigned long long>(fnv1a(src)),
                static_cast<unsigned long long>(headers_hash), major, minor);
  const std::string key = std::string(hx) + "@" + std::to_string(dev);
  auto it = g_functions.find(key);
  if (it != g_functions.end()) return it->second;
  auto f = g_failed.find(key);
  if (f != g_failed.end()) {
    *why = f->second;
    return nullptr;
  }
  std::vector<char> cubin;
  const std::string dir = cache_dir();
  const std::string path = dir + "/" + hx + ".cubin";
  {
    std::ifstream in(path, std::ios::binary);
    if (in) cubin.assign(std::istreambuf_iterator<char>(in), std::istreambuf_iterator<char>());
  }
  if (cubin.empty()) {
    if (!compile_cubin(src, &cubin, why)) {
      g_failed[key] = *why;
      return nullptr;
    }
    mkdirs(dir);
    const std::string tmp = path + ".tmp" + std::to_string(getpid());
    {
      std::ofstream out(tmp, std::ios::binary);
      out.write(cubin.data(), std::streamsize(cubin.size()));
    }
    std::rename(tmp.c_str(), path.c_str());
  }
  cudaFree(nullptr);  // make sure the runtime's primary context is current
  CUmodule mod;
  CUfunction fn;
  if (A.moduleLoadData(&mod, cubin.data()) != CUDA_SUCCESS || A.moduleGetFunction(&fn, mod, kernel_name(kind)) != CUDA_SUCCESS) {
    *why = "loading the compiled module failed";
    g_failed[key] = *why;
    return nullptr;
  }
  g_functions[key] = fn;
  return fn;
}

}  // namespace

// How forward dynamics is computed in the specialised sweep: 0 automatic (the route with the
// smaller FP64 operation count for this model and op set), 1 the articulated-body passes, 2
// from the mass matrix (OP_FD_CRBA).
std::atomic<int> g_fd_method{0};

// Estimated FP64 operations of the two routes (counted from the sweep's source: per 1-DoF
// joint the articulated-body passes take ~205, a root free flyer ~550 and another ~1400;
// the mass-matrix route needs the composite inertias and the zero-acceleration forces when
// the op set does not already compute them, the L^T D L factorisation (a reciprocal per
// column and, per ancestor c of a column, depth(c) + 2), the solve (2 depth + 2 per column)
// and, with inverse dynamics requested, M qdd (2 depth + 1 per column)).
bool fd_by_mass_matrix(const Model& M, int ops) {
  if (!(ops & OP_ABA)) return false;
  const auto& t = M.host_table();
  const auto* hdr = reinterpret_cast<const DModel*>(t.data());
  const DJoint* J = model_joints(hdr);
  const int nj = hdr->nj, nv = hdr->nv;
  // ancestor columns per column (no allocation: this runs on every host-path call); the
  // route needs parents numbered before children
  int depth[kMaxTreeColumns];
  if (nv > kMaxTreeColumns) return false;
  for (int i = 1; i < nj; i++) {
    const int p = J[i].parent;
    if (p > 0 && J[p].ivx + J[p].nv > J[i].ivx) return false;
    const int base = p > 0 ? depth[J[p].ivx + J[p].nv - 1] + 1 : 0;
    for (int k = 0; k < J[i].nv; k++) depth[J[i].ivx + k] = base + k;
  }
  const int mode = g_fd_method.load();
  if (mode != 0) return mode == 2;
  double art = 0, mm = 0;
  for (int i = 1; i < nj; i++) {
    art += J[i].nv == 1 ? 205 : (J[i].parent == 0 ? 550 : 1400);
    if (!(ops & OP_CRBA)) mm += 10;
    if (!(ops & OP_RNEA)) mm += 60;
  }
  for (int a = 0; a < nv; a++) {
    const int d = depth[a];
    if (!(ops & OP_CRBA)) mm += 24 + 6 * (d + 1);
    mm += 5 + 2 * d + 2;                // reciprocal, solve
    if (ops & OP_RNEA) mm += 2 * d + 1;  // M qdd
    // factorisation: column a updates, for each ancestor c (depths d-1 .. 0), c's row over
    // c and its ancestors
    mm += double(d) * (d - 1) / 2 + 2.0 * d;
  }
  return mm < art;
}

int step_kernel_ops(const Model& M, int ops) { return fd_by_mass_matrix(M, ops) ? ops | OP_FD_CRBA : ops; }

void fd_method(int mode, int* out) {
  if (mode >= 0) g_fd_method.store(mode);
  if (out) *out = g_fd_method.load();
}

std::string step_jit_source(const Model& M, int ops) {
  return generate_source(M, JIT_STEP, step_kernel_ops(M, ops));
}
std::string rollout_jit_source(const Model& M) {
  return generate_source(M, JIT_ROLLOUT_FWD, 0);
}

void set_jit_config(int enable, int64_t min_n) {
  std::lock_guard<std::mutex> lk(g_mu);
  read_env_config();
  if (enable >= 0) g_enable = enable ? 1 : 0;
  if (min_n >= 0) g_min_n = min_n;
}

void get_jit_config(int* enable, int64_t* min_n) {
  std::lock_guard<std::mutex> lk(g_mu);
  read_env_config();
  if (enable) *enable = g_enable;
  if (min_n) *min_n = g_min_n;
}

void jit_max_joints(int max_joints, int* out) {
  std::lock_guard<std::mutex> lk(g_mu);
  read_env_config();
  if (max_joints >= 0) g_max_joints = max_joints;
  if (out) *out = g_max_joints;
}

bool prepare_step_jit(Model& M, int ops, std::string* why) {
  std::lock_guard<std::mutex> lk(g_mu);
  read_env_config();
  return get_function(M, JIT_STEP, step_kernel_ops(M, ops), why) != nullptr;
}

bool prepare_rollout_jit(Model& M, std::string* why) {
  std::lock_guard<std::mutex> lk(g_mu);
  read_env_config();
  return get_function(M, JIT_ROLLOUT_FWD, 0, why) != nullptr;
}

namespace {
template <class Args>
bool launch_jit(Model& M, int kind, int ops, const Args& a, cudaStream_t s, std::string* why, int joints = -1,
                int threads = 32) {
  CUfunction fn;
  {
    std::lock_guard<std::mutex> lk(g_mu);
    read_env_config();
    if (!g_enable) {
      *why = "disabled";
      return false;
    }
    if (a.n < g_min_n) {
      *why = "batch below the run-time compilation threshold";
      return false;
    }
    if ((joints >= 0 ? joints : M.njoints()) > g_max_joints) {
      *why = "tree above the run-time compilation size limit";
      return false;
    }
    fn = get_function(M, kind, ops, why);
  }
  if (!fn) return false;
  Args args = a;
  void* params[] = {&args};
  const int per = envs_per_block(kind);
  const unsigned blocks = unsigned((a.n + per - 1) / per);
  if (api().launchKernel(fn, blocks, 1, 1, unsigned(threads), 1, 1, 0, reinterpret_cast<CUstream>(s), params,
                         nullptr) != CUDA_SUCCESS) {
    *why = "cuLaunchKernel failed";
    return false;
  }
  return true;
}
}  // namespace

bool launch_step_jit(Model& M, int ops, const StepArgs& a, cudaStream_t s, std::string* why) {
  return launch_jit(M, JIT_STEP, step_kernel_ops(M, ops), a, s, why);
}

namespace {
// The size limit applies to what one warp sweeps: the trunk and the longest role.
int role_joints(const Model& M, int lanes) {
  const std::vector<int> tt = M.team_table(lanes);
  return 1 + tt[1] + tt[2];
}

CUfunction roles_function(Model& M, int lanes, int ops, int64_t n, std::string* why) {
  std::lock_guard<std::mutex> lk(g_mu);
  read_env_config();
  if (!g_enable) {
    *why = "disabled";
    return nullptr;
  }
  if (n < g_min_n) {
    *why = "batch below the run-time compilation threshold";
    return nullptr;
  }
  if (role_joints(M, lanes) > g_max_joints) {
    *why = "tree above the run-time compilation size limit";
    return nullptr;
  }
  return get_function(M, JIT_STEP_ROLES, ops | (lanes << kRoleLanesShift), why);
}

bool launch_roles(CUfunction fn, int lanes, const StepArgs& a, const int* rows, int64_t count, double dt,
                  int integrate, cudaStream_t s, std::string* why) {
  StepArgs args = a;
  long long cnt = count;
  void* params[] = {&args, &rows, &cnt, &dt, &integrate};
  if (api().launchKernel(fn, unsigned((count + 31) / 32), 1, 1, unsigned(32 * lanes), 1, 1, 0,
                         reinterpret_cast<CUstream>(s), params, nullptr) != CUDA_SUCCESS) {
    *why = "cuLaunchKernel failed";
    return false;
  }
  return true;
}

}  // namespace

bool launch_step_roles_jit(Model& M, int lanes, int ops, const StepArgs& a, cudaStream_t s, std::string* why) {
  CUfunction fn = roles_function(M, lanes, ops, a.n, why);
  return fn && launch_roles(fn, lanes, a, nullptr, a.n, 0.0, 0, s, why);
}

bool step_roles_jit_ready(Model& M, int lanes, int ops, int64_t n, std::string* why) {
  return roles_function(M, lanes, ops, n, why) != nullptr;
}

bool launch_step_roles_rows_jit(Model& M, int lanes, int ops, const StepArgs& a, const int* rows, int64_t count,
                                double dt, bool integrate, cudaStream_t s, std::string* why) {
  // (the batch-size threshold was applied to the whole batch by step_roles_jit_ready)
  CUfunction fn = roles_function(M, lanes, ops, INT64_MAX, why);
  return fn && launch_roles(fn, lanes, a, rows, count, dt, integrate ? 1 : 0, s, why);
}

bool prepare_step_roles_jit(Model& M, int lanes, int ops, std::string* why) {
  std::lock_guard<std::mutex> lk(g_mu);
  read_env_config();
  return get_function(M, JIT_STEP_ROLES, ops | (lanes << kRoleLanesShift), why) != nullptr;
}

std::string step_roles_jit_source(const Model& M, int lanes, int ops) {
  return generate_source(M, JIT_STEP_ROLES, ops | (lanes << kRoleLanesShift));
}

bool launch_rollout_jit(Model& M, const RolloutArgs& a, cudaStream_t s, std::string* why) {
  return launch_jit(M, JIT_ROLLOUT_FWD, 0, a, s, why);
}

bool launch_rollout3_jit(Model& M, const RolloutArgs& a, cudaStream_t s, std::string* why) {
  return launch_jit(M, JIT_ROLLOUT_FWD3, 0, a, s, why);
}

bool launch_rollout_reverse3_jit(Model& M, const RolloutArgs& a, cudaStream_t s, std::string* why) {
  return launch_jit(M, JIT_ROLLOUT_REV3, 0, a, s, why);
}

bool launch_aba3_jit(Model& M, const StepArgs& a, cudaStream_t s, std::string* why) {
  return launch_jit(M, JIT_ABA3, 0, a, s, why);
}

std::string aba3_jit_source(const Model& M) { return generate_source(M, JIT_ABA3, 0); }

bool prepare_aba3_jit(Model& M, std::string* why) {
  std::lock_guard<std::mutex> lk(g_mu);
  read_env_config();
  return get_function(M, JIT_ABA3, 0, why) != nullptr;
}

std::string rollout3_jit_source(const Model& M, bool reverse) {
  return generate_source(M, reverse ? JIT_ROLLOUT_REV3 : JIT_ROLLOUT_FWD3, 0);
}

bool prepare_rollout3_jit(Model& M, bool reverse, std::string* why) {
  std::lock_guard<std::mutex> lk(g_mu);
  read_env_config();
  return get_function(M, reverse ? JIT_ROLLOUT_REV3 : JIT_ROLLOUT_FWD3, 0, why) != nullptr;
}

bool launch_vjp_jit(Model& M, bool aba, const VjpArgs& a, cudaStream_t s, std::string* why) {
  return launch_jit(M, aba ? JIT_ABA_VJP : JIT_RNEA_VJP, 0, a, s, why);
}

std::string vjp_jit_source(const Model& M, bool aba) { return generate_source(M, aba ? JIT_ABA_VJP : JIT_RNEA_VJP, 0); }

bool prepare_vjp_jit(Model& M, bool aba, std::string* why) {
  std::lock_guard<std::mutex> lk(g_mu);
  read_env_config();
  return get_function(M, aba ? JIT_ABA_VJP : JIT_RNEA_VJP, 0, why) != nullptr;
}

}  // namespace sgdyn
