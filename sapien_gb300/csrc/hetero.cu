// Heterogeneous batches: robots of different size and topology in one persistent launch.
//
// Plan (host, once per batch): the models' tables are packed into one device buffer;
// environments are grouped per model into tiles of up to 32 (one warp each); tiles are
// ordered by descending velocity dimension (longest work first), so the largest trees
// start first and small ones fill in behind them.
// Step (device): a persistent grid of warps pulls tile indices from a global counter with
// atomicAdd until the queue is exhausted; each lane runs the fused sweep for one
// environment with its own model's table, or, for a model given L lanes per environment,
// each team of L lanes shares one environment (trunk + branches, see step_kernel.cuh) and
// a tile holds 32 / L environments. No warp ever waits on another, so there is no
// spin loop to bound. The counter is reset with cudaMemsetAsync on the same stream before
// every launch, which keeps a step stream-ordered and capturable into a CUDA graph.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>
#include <numeric>
#include <stdexcept>
#include <string>
#include <vector>

#include "../../include/sgdyn.h"
#include "trace.h"
#include "jit.h"
#include "model.h"
#include "se3.cuh"
#include "step_kernel.cuh"

struct sgdyn_model {
  sgdyn::Model* impl;
};

namespace sgdyn {

int set_last_error(int code, const std::string& msg);

struct HeteroArgs {
  const unsigned char* tables;
  const int64_t* table_offset;
  const int* teams;             // team tables of the models run with L > 1
  const int64_t* team_offset;   // per model (-1: one lane per environment)
  const int* perm;
  const int4* tiles;  // (model, start, count, lanes per environment)
  int ntiles;
  unsigned int* head;
  // per-model byte sizes of the packed tables and int counts of the team tables; each warp
  // stages its tile's tables in its slice of the dynamic shared memory (stage_bytes each:
  // the largest model table, then the largest team table)
  const int* table_bytes;
  const int* team_ints;
  int stage_bytes, stage_team_at;
  StepArgs io;
  // semi-implicit Euler after the sweep (integrate != 0): q / qd rows updated in place
  int integrate;
  double dt;
  double* q_state;
  double* qd_state;
};

// qd += dt qdd, then q advanced by dt qd on one environment's padded rows (angles and
// slides add; a free flyer moves on SE(3) by its body twist).
__device__ __forceinline__ void integrate_env(const DModel* m, double* q, double* qd, const double* qdd, double dt) {
  integrate_env_t(RuntimeTab{m}, q, qd, qdd, dt);
}

template <int MAXJ, int OPS>
__global__ void hetero_kernel(const HeteroArgs a) {
  extern __shared__ __align__(16) unsigned char stage[];
  const int lane = threadIdx.x & 31;
  unsigned char* const mine = stage + int64_t(threadIdx.x >> 5) * a.stage_bytes;
  const DModel* m = reinterpret_cast<const DModel*>(mine);
  const int* team = reinterpret_cast<const int*>(mine + a.stage_team_at);
  int staged = -1;  // model whose tables this warp holds
  for (;;) {
    unsigned t = 0;
    if (lane == 0) t = atomicAdd(a.head, 1u);
    t = __shfl_sync(0xffffffffu, t, 0);
    if (t >= unsigned(a.ntiles)) break;
    const int4 tile = a.tiles[t];
    if (tile.x != staged) {
      // the sweeps read the model's joint and link tables (and the team table) over and
      // over; from shared memory those reads do not compete with the sweep's local-memory
      // working set in L1
      __syncwarp();
      const int4* src = reinterpret_cast<const int4*>(a.tables + a.table_offset[tile.x]);
      int4* dst = reinterpret_cast<int4*>(mine);
      for (int k = lane; k < a.table_bytes[tile.x] / 16; k += 32) dst[k] = src[k];
      if (a.team_offset[tile.x] >= 0) {
        int* tdst = reinterpret_cast<int*>(mine + a.stage_team_at);
        const int* tsrc = a.teams + a.team_offset[tile.x];
        for (int k = lane; k < a.team_ints[tile.x]; k += 32) tdst[k] = tsrc[k];
      }
      __syncwarp();
      staged = tile.x;
    }
    if (tile.w <= 1) {
      if (lane < tile.z) step_env<MAXJ, OPS>(m, a.io, int64_t(a.perm[tile.y + lane]));
    } else {
      // every lane takes part (the team sums are warp shuffles); lanes of an empty tail
      // slot repeat the tile's first environment and store nothing
      const int slot = lane / tile.w;
      const bool valid = slot < tile.z;
      const TeamLanes tm{team, lane % tile.w, valid};
      step_env_t<MAXJ, OPS>(RuntimeTab{m}, a.io, int64_t(a.perm[tile.y + (valid ? slot : 0)]), tm);
    }
    if (a.integrate) {
      // the sweep's reads of q / qd and writes of qdd are done on every lane of the tile;
      // one lane per environment then integrates it
      __syncwarp();
      const int w = tile.w <= 1 ? 1 : tile.w;
      if (lane % w == 0 && lane / w < tile.z) {
        const int64_t env = a.perm[tile.y + lane / w];
        integrate_env(m, a.q_state + env * a.io.q.es, a.qd_state + env * a.io.qd.es,
                      a.io.qdd_out.p + env * a.io.qdd_out.es, a.dt);
      }
    }
    __syncwarp();
  }
}

// Semi-implicit Euler on padded env-major rows: qd += dt qdd, then q (+)= dt qd with each
// environment's own model (angles and slides add; a free flyer moves on SE(3) by its body
// twist). A block of kIntegrateThreads threads takes 32 consecutive environments, whose
// padded rows form one contiguous block: its threads walk the flat (environment, joint)
// pairs, each one-DoF joint updating its velocity and position in one go, and the first
// warp then moves the free flyers, lane i those of environment i, so the exponential map
// runs SIMD across environments. Every joint's columns are written by one thread only.
constexpr int kIntegrateThreads = 128;

struct HeteroIntegrateArgs {
  const unsigned char* tables;
  const int64_t* table_offset;
  const int* model_of_env;
  int64_t n;
  int max_nq, max_nv, joints;  // joints: moving-joint slots per environment (max njoints - 1)
  double dt;
  double* q;
  double* qd;
  const double* qdd;
};

__global__ void __launch_bounds__(kIntegrateThreads) hetero_integrate_kernel(const HeteroIntegrateArgs a) {
  __shared__ const DModel* models[32];
  const int64_t e0 = int64_t(blockIdx.x) * 32;
  const int envs = a.n - e0 < 32 ? int(a.n - e0) : 32;
  if (threadIdx.x < envs)
    models[threadIdx.x] = reinterpret_cast<const DModel*>(a.tables + a.table_offset[a.model_of_env[e0 + threadIdx.x]]);
  __syncthreads();
  double* __restrict__ Q = a.q + e0 * a.max_nq;
  double* __restrict__ QD = a.qd + e0 * a.max_nv;
  const double* __restrict__ QDD = a.qdd + e0 * a.max_nv;
  const double dt = a.dt;
#pragma unroll 4
  for (int k = threadIdx.x; k < envs * a.joints; k += kIntegrateThreads) {
    const int el = k / a.joints, i = 1 + (k - el * a.joints);
    const DModel* m = models[el];
    if (i >= m->nj) continue;
    const DJoint& J = model_joints(m)[i];
    if (J.kind == JK_FREEFLYER) continue;
    const int64_t c = int64_t(el) * a.max_nv + J.vcol;
    const double w = fma(dt, QDD[c], QD[c]);
    QD[c] = w;
    double& qc = Q[int64_t(el) * a.max_nq + J.qcol];
    qc = fma(dt, w, qc);
  }
  if (threadIdx.x >= envs) return;
  const DModel* m = models[threadIdx.x];
  const DJoint* JT = model_joints(m);
  for (int i = 1; i < m->nj; i++) {
    if (JT[i].kind != JK_FREEFLYER) continue;
    const int64_t c = int64_t(threadIdx.x) * a.max_nv + JT[i].vcol;
    double v[6];
#pragma unroll
    for (int k = 0; k < 6; k++) {
      const double w = fma(dt, QDD[c + k], QD[c + k]);
      QD[c + k] = w;
      v[k] = dt * w;
    }
    free_flyer_integrate(Q + int64_t(threadIdx.x) * a.max_nq + JT[i].qcol, v);
  }
}

template <int MAXJ>
cudaError_t launch_hetero_bucket(int ops, const HeteroArgs& a, dim3 grid, dim3 block, cudaStream_t s) {
  const size_t smem = size_t(a.stage_bytes) * (block.x / 32);
  switch (ops) {
#define SG_CASE(O)                                                                                            \
  case O:                                                                                                     \
    if (smem > 48 * 1024 &&                                                                                   \
        cudaFuncSetAttribute(hetero_kernel<MAXJ, O>, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem)) != \
            cudaSuccess)                                                                                      \
      return cudaErrorInvalidValue;                                                                           \
    hetero_kernel<MAXJ, O><<<grid, block, smem, s>>>(a);                                                      \
    break;
    SG_CASE(OP_CRBA | OP_RNEA | OP_ABA)
    SG_CASE(OP_RNEA | OP_ABA)
    SG_CASE(OP_ALL)
    SG_CASE(OP_RNEA)
    SG_CASE(OP_ABA)
    SG_CASE(OP_CRBA)
#undef SG_CASE
    default: return cudaErrorInvalidValue;
  }
  return cudaGetLastError();
}

}  // namespace sgdyn

using namespace sgdyn;

struct sgdyn_batch {
  std::vector<const sgdyn_model*> models;
  int64_t n = 0;
  int max_nq = 0, max_nv = 0, max_nlinks = 0, max_nj = 0;
  std::vector<int> model_of_env;
  std::vector<int> lanes;  // lanes per environment, per model
  // device
  unsigned char* tables = nullptr;
  int64_t* offsets = nullptr;
  int* table_bytes = nullptr;  // per model, rounded up to 16
  int* team_ints = nullptr;    // per model (0 with one lane per environment)
  int max_table_bytes = 0, max_team_ints = 0;
  int* teams = nullptr;
  int64_t* team_offsets = nullptr;
  int* model_of_env_dev = nullptr;
  int* perm = nullptr;
  int4* tiles = nullptr;
  int ntiles = 0;
  // the models run with teams can take the specialised one-warp-per-role sweep (a launch
  // each, beside the persistent kernel, which then takes the other models' tiles only)
  int* model_rows = nullptr;  // environments of each model, model after model
  std::vector<int64_t> model_row_start, model_row_count;
  int4* rest_tiles = nullptr;  // the tiles of the models with one lane per environment
  int nrest = 0;
  std::vector<cudaStream_t> side;
  unsigned int* head = nullptr;
  int device = -1;
  // launch shape (autotuned)
  int ctas_per_sm = 4, warps_per_cta = 1, order = 0;
  int sms = 0;
};

namespace {

void free_device(sgdyn_batch* b) {
  cudaFree(b->tables);
  cudaFree(b->offsets);
  cudaFree(b->table_bytes);
  cudaFree(b->team_ints);
  b->table_bytes = nullptr;
  b->team_ints = nullptr;
  cudaFree(b->teams);
  cudaFree(b->team_offsets);
  cudaFree(b->model_of_env_dev);
  b->teams = nullptr;
  b->team_offsets = nullptr;
  b->model_of_env_dev = nullptr;
  cudaFree(b->perm);
  cudaFree(b->tiles);
  cudaFree(b->head);
  cudaFree(b->model_rows);
  cudaFree(b->rest_tiles);
  b->model_rows = nullptr;
  b->rest_tiles = nullptr;
  b->tables = nullptr;
  b->offsets = nullptr;
  b->perm = nullptr;
  b->tiles = nullptr;
  b->head = nullptr;
}

// Builds the permutation and tile list for the current order and uploads them.
int upload_plan(sgdyn_batch* b) {
  const int nm = int(b->models.size());
  std::vector<std::vector<int>> envs(nm);
  for (int64_t e = 0; e < b->n; e++) envs[b->model_of_env[e]].push_back(int(e));
  std::vector<int> mo(nm);
  std::iota(mo.begin(), mo.end(), 0);
  if (b->order == 0)
    std::stable_sort(mo.begin(), mo.end(),
                     [&](int x, int y) { return b->models[x]->impl->nv() > b->models[y]->impl->nv(); });
  std::vector<int> perm;
  std::vector<int4> tiles;
  if (b->order == 0) {
    for (int m : mo) {
      const size_t per_tile = size_t(32 / b->lanes[m]);
      for (size_t s = 0; s < envs[m].size(); s += per_tile) {
        int cnt = int(std::min<size_t>(per_tile, envs[m].size() - s));
        tiles.push_back(make_int4(m, int(perm.size()), cnt, b->lanes[m]));
        for (int k = 0; k < cnt; k++) perm.push_back(envs[m][s + k]);
      }
    }
  } else {
    // input order: consecutive environments of the same model share a tile
    int64_t e = 0;
    while (e < b->n) {
      int m = b->model_of_env[e];
      const int per_tile = 32 / b->lanes[m];
      int cnt = 0;
      int start = int(perm.size());
      while (e < b->n && cnt < per_tile && b->model_of_env[e] == m) {
        perm.push_back(int(e));
        e++;
        cnt++;
      }
      tiles.push_back(make_int4(m, start, cnt, b->lanes[m]));
    }
  }
  std::vector<int> rows;
  b->model_row_start.assign(nm, 0);
  b->model_row_count.assign(nm, 0);
  for (int m = 0; m < nm; m++) {
    b->model_row_start[m] = int64_t(rows.size());
    b->model_row_count[m] = int64_t(envs[m].size());
    rows.insert(rows.end(), envs[m].begin(), envs[m].end());
  }
  std::vector<int4> rest;
  for (const int4& t : tiles)
    if (t.w <= 1) rest.push_back(t);
  cudaFree(b->perm);
  cudaFree(b->tiles);
  cudaFree(b->model_rows);
  cudaFree(b->rest_tiles);
  b->perm = nullptr;
  b->tiles = nullptr;
  b->model_rows = nullptr;
  b->rest_tiles = nullptr;
  if (cudaMalloc(&b->perm, sizeof(int) * std::max<size_t>(perm.size(), 1)) != cudaSuccess ||
      cudaMalloc(&b->tiles, sizeof(int4) * std::max<size_t>(tiles.size(), 1)) != cudaSuccess ||
      cudaMalloc(&b->model_rows, sizeof(int) * std::max<size_t>(rows.size(), 1)) != cudaSuccess ||
      cudaMalloc(&b->rest_tiles, sizeof(int4) * std::max<size_t>(rest.size(), 1)) != cudaSuccess)
    return SGDYN_ERR_CUDA;
  if (!rows.empty() && cudaMemcpy(b->model_rows, rows.data(), sizeof(int) * rows.size(), cudaMemcpyHostToDevice) !=
                           cudaSuccess)
    return SGDYN_ERR_CUDA;
  if (!rest.empty() &&
      cudaMemcpy(b->rest_tiles, rest.data(), sizeof(int4) * rest.size(), cudaMemcpyHostToDevice) != cudaSuccess)
    return SGDYN_ERR_CUDA;
  b->nrest = int(rest.size());
  if (!perm.empty() && cudaMemcpy(b->perm, perm.data(), sizeof(int) * perm.size(), cudaMemcpyHostToDevice) != cudaSuccess)
    return SGDYN_ERR_CUDA;
  if (!tiles.empty() &&
      cudaMemcpy(b->tiles, tiles.data(), sizeof(int4) * tiles.size(), cudaMemcpyHostToDevice) != cudaSuccess)
    return SGDYN_ERR_CUDA;
  b->ntiles = int(tiles.size());
  return SGDYN_OK;
}

int upload_teams(sgdyn_batch* b) {
  std::vector<int> all, counts;
  std::vector<int64_t> offs;
  for (size_t m = 0; m < b->models.size(); m++) {
    if (b->lanes[m] <= 1) {
      offs.push_back(-1);
      counts.push_back(0);
      continue;
    }
    offs.push_back(int64_t(all.size()));
    const auto t = b->models[m]->impl->team_table(b->lanes[m]);
    all.insert(all.end(), t.begin(), t.end());
    counts.push_back(int(t.size()));
  }
  b->max_team_ints = counts.empty() ? 0 : *std::max_element(counts.begin(), counts.end());
  cudaFree(b->teams);
  cudaFree(b->team_offsets);
  cudaFree(b->team_ints);
  b->teams = nullptr;
  b->team_offsets = nullptr;
  b->team_ints = nullptr;
  if (cudaMalloc(&b->teams, sizeof(int) * std::max<size_t>(all.size(), 1)) != cudaSuccess ||
      cudaMalloc(&b->team_offsets, sizeof(int64_t) * offs.size()) != cudaSuccess ||
      cudaMalloc(&b->team_ints, sizeof(int) * counts.size()) != cudaSuccess ||
      cudaMemcpy(b->team_ints, counts.data(), sizeof(int) * counts.size(), cudaMemcpyHostToDevice) != cudaSuccess)
    return SGDYN_ERR_CUDA;
  if (!all.empty() && cudaMemcpy(b->teams, all.data(), sizeof(int) * all.size(), cudaMemcpyHostToDevice) != cudaSuccess)
    return SGDYN_ERR_CUDA;
  if (cudaMemcpy(b->team_offsets, offs.data(), sizeof(int64_t) * offs.size(), cudaMemcpyHostToDevice) != cudaSuccess)
    return SGDYN_ERR_CUDA;
  return SGDYN_OK;
}

bool dev_ptr(const void* p) { return device_accessible(p); }

Arr env_major(const void* p, int64_t cols) { return Arr{static_cast<double*>(const_cast<void*>(p)), cols, 1}; }

}  // namespace

extern "C" {

int sgdyn_batch_create(const sgdyn_model* const* models, int nmodels, const int* model_of_env, int64_t n,
                       sgdyn_batch** out) {
  if (!models || nmodels <= 0 || !out || (n > 0 && !model_of_env))
    return set_last_error(SGDYN_ERR_NULL, "null argument");
  if (n < 0 || n > int64_t(1) << 31) return set_last_error(SGDYN_ERR_RUNTIME, "bad batch size");
  auto* b = new sgdyn_batch;
  b->n = n;
  for (int k = 0; k < nmodels; k++) {
    if (!models[k] || !models[k]->impl) {
      delete b;
      return set_last_error(SGDYN_ERR_NULL, "null model in batch");
    }
    const Model& M = *models[k]->impl;
    int nff = 0;
    for (auto& J : M.joints) nff += J.kind == JK_FREEFLYER;
    if (nff > 1 || stash_bucket(M.njoints()) == 0 || M.njoints() > 32) {
      delete b;
      return set_last_error(SGDYN_ERR_UNSUPPORTED, "batch models need at most 31 moving joints and one free flyer");
    }
    b->models.push_back(models[k]);
    b->max_nq = std::max(b->max_nq, M.nq_ext());
    b->max_nv = std::max(b->max_nv, M.nv());
    b->max_nlinks = std::max(b->max_nlinks, M.nlinks());
    b->max_nj = std::max(b->max_nj, M.njoints());
  }
  b->model_of_env.assign(model_of_env, model_of_env + n);
  b->lanes.assign(b->models.size(), 1);
  for (int m : b->model_of_env)
    if (m < 0 || m >= nmodels) {
      delete b;
      return set_last_error(SGDYN_ERR_RUNTIME, "model index out of range");
    }
  cudaGetDevice(&b->device);
  cudaDeviceGetAttribute(&b->sms, cudaDevAttrMultiProcessorCount, b->device);
  // pack tables (16-byte aligned offsets)
  std::vector<unsigned char> packed;
  std::vector<int64_t> offs;
  std::vector<int> sizes;
  for (auto* m : b->models) {
    const auto& t = m->impl->host_table();
    offs.push_back(int64_t(packed.size()));
    sizes.push_back(int((t.size() + 15) / 16 * 16));
    packed.insert(packed.end(), t.begin(), t.end());
    while (packed.size() % 256) packed.push_back(0);
  }
  b->max_table_bytes = *std::max_element(sizes.begin(), sizes.end());
  if (cudaMalloc(&b->tables, packed.size()) != cudaSuccess ||
      cudaMalloc(&b->offsets, sizeof(int64_t) * offs.size()) != cudaSuccess ||
      cudaMalloc(&b->table_bytes, sizeof(int) * sizes.size()) != cudaSuccess ||
      cudaMemcpy(b->table_bytes, sizes.data(), sizeof(int) * sizes.size(), cudaMemcpyHostToDevice) != cudaSuccess ||
      cudaMalloc(&b->head, sizeof(unsigned int)) != cudaSuccess ||
      cudaMemcpy(b->tables, packed.data(), packed.size(), cudaMemcpyHostToDevice) != cudaSuccess ||
      cudaMemcpy(b->offsets, offs.data(), sizeof(int64_t) * offs.size(), cudaMemcpyHostToDevice) != cudaSuccess ||
      cudaMalloc(&b->model_of_env_dev, sizeof(int) * std::max<int64_t>(n, 1)) != cudaSuccess ||
      (n > 0 && cudaMemcpy(b->model_of_env_dev, b->model_of_env.data(), sizeof(int) * n, cudaMemcpyHostToDevice) !=
                    cudaSuccess) ||
      upload_teams(b) != SGDYN_OK || upload_plan(b) != SGDYN_OK) {
    free_device(b);
    delete b;
    return set_last_error(SGDYN_ERR_CUDA, "batch upload failed");
  }
  *out = b;
  return SGDYN_OK;
}

void sgdyn_batch_free(sgdyn_batch* b) {
  if (!b) return;
  free_device(b);
  for (cudaStream_t st : b->side)
    if (st) cudaStreamDestroy(st);
  delete b;
}

int sgdyn_batch_info(const sgdyn_batch* b, int64_t* n, int* max_nq, int* max_nv, int* max_nlinks) {
  if (!b) return set_last_error(SGDYN_ERR_NULL, "null batch");
  if (n) *n = b->n;
  if (max_nq) *max_nq = b->max_nq;
  if (max_nv) *max_nv = b->max_nv;
  if (max_nlinks) *max_nlinks = b->max_nlinks;
  return SGDYN_OK;
}

int sgdyn_batch_set_launch(sgdyn_batch* b, int ctas_per_sm, int warps_per_cta, int order) {
  if (!b) return set_last_error(SGDYN_ERR_NULL, "null batch");
  if (ctas_per_sm < 1 || ctas_per_sm > 32 || warps_per_cta < 1 || warps_per_cta > 8 || order < 0 || order > 1)
    return set_last_error(SGDYN_ERR_RUNTIME, "bad launch shape");
  b->ctas_per_sm = ctas_per_sm;
  b->warps_per_cta = warps_per_cta;
  if (order != b->order) {
    b->order = order;
    if (upload_plan(b) != SGDYN_OK) return set_last_error(SGDYN_ERR_CUDA, "plan upload failed");
  }
  return SGDYN_OK;
}

int sgdyn_batch_set_lanes(sgdyn_batch* b, const int* lanes_per_model) {
  if (!b || !lanes_per_model) return set_last_error(SGDYN_ERR_NULL, "null argument");
  for (size_t m = 0; m < b->models.size(); m++) {
    const int L = lanes_per_model[m];
    if (L != 1 && L != 2 && L != 4 && L != 8) return set_last_error(SGDYN_ERR_RUNTIME, "lanes must be 1, 2, 4 or 8");
  }
  b->lanes.assign(lanes_per_model, lanes_per_model + b->models.size());
  if (upload_teams(b) != SGDYN_OK || upload_plan(b) != SGDYN_OK)
    return set_last_error(SGDYN_ERR_CUDA, "team / plan upload failed");
  return SGDYN_OK;
}

int sgdyn_batch_integrate(sgdyn_batch* b, double dt, double* q, double* qd, const double* qdd, void* stream) {
  SG_TRACE("sgdyn_batch_integrate");
  if (!b) return set_last_error(SGDYN_ERR_NULL, "null batch");
  if (b->n == 0) return SGDYN_OK;
  if (!dev_ptr(q) || !dev_ptr(qd) || !dev_ptr(qdd))
    return set_last_error(SGDYN_ERR_NULL, "q / qd / qdd is null or not device memory");
  if (!b->model_of_env_dev) return set_last_error(SGDYN_ERR_RUNTIME, "batch has no environment table");
  HeteroIntegrateArgs a;
  a.tables = b->tables;
  a.table_offset = b->offsets;
  a.model_of_env = b->model_of_env_dev;
  a.n = b->n;
  a.max_nq = b->max_nq;
  a.max_nv = b->max_nv;
  a.joints = b->max_nj - 1;
  a.dt = dt;
  a.q = q;
  a.qd = qd;
  a.qdd = qdd;
  if (a.joints <= 0 || b->n == 0) return SGDYN_OK;
  hetero_integrate_kernel<<<unsigned((b->n + 31) / 32), kIntegrateThreads, 0, static_cast<cudaStream_t>(stream)>>>(a);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return set_last_error(SGDYN_ERR_CUDA, std::string("kernel launch failed: ") + cudaGetErrorString(e));
  return SGDYN_OK;
}

static int batch_step(sgdyn_batch* b, int ops, const double* q, const double* qd, const double* qdd, const double* tau,
                      double* link_poses, double* J, double* M, double* tau_out, double* qdd_out, void* stream,
                      bool integrate, double dt) {
  if (!b) return set_last_error(SGDYN_ERR_NULL, "null batch");
  if (b->n == 0) return SGDYN_OK;
  if (!dev_ptr(q)) return set_last_error(SGDYN_ERR_NULL, "q is null or not device memory");
  if ((ops & (OP_RNEA | OP_ABA)) && !dev_ptr(qd)) return set_last_error(SGDYN_ERR_NULL, "qd missing");
  if ((ops & OP_RNEA) && (!dev_ptr(qdd) || !dev_ptr(tau_out))) return set_last_error(SGDYN_ERR_NULL, "qdd / tau_out missing");
  if ((ops & OP_ABA) && (!dev_ptr(tau) || !dev_ptr(qdd_out))) return set_last_error(SGDYN_ERR_NULL, "tau / qdd_out missing");
  if ((ops & OP_CRBA) && !dev_ptr(M)) return set_last_error(SGDYN_ERR_NULL, "M missing");
  if ((ops & OP_FK) && !dev_ptr(link_poses)) return set_last_error(SGDYN_ERR_NULL, "link_poses missing");
  if ((ops & OP_JAC) && !dev_ptr(J)) return set_last_error(SGDYN_ERR_NULL, "J missing");
  const int64_t nv = b->max_nv;
  HeteroArgs a;
  a.tables = b->tables;
  a.table_offset = b->offsets;
  a.teams = b->teams;
  a.team_offset = b->team_offsets;
  a.table_bytes = b->table_bytes;
  a.team_ints = b->team_ints;
  a.stage_team_at = b->max_table_bytes;
  a.stage_bytes = (b->max_table_bytes + 4 * b->max_team_ints + 15) / 16 * 16;
  a.perm = b->perm;
  a.tiles = b->tiles;
  a.ntiles = b->ntiles;
  a.head = b->head;
  a.io.n = b->n;
  a.io.q = env_major(q, b->max_nq);
  a.io.qd = env_major(qd, nv);
  a.io.qdd = env_major(qdd, nv);
  a.io.tau = env_major(tau, nv);
  a.io.poses = env_major(link_poses, int64_t(b->max_nlinks) * 7);
  a.io.J = env_major(J, 6 * nv);
  a.io.M = env_major(M, nv * nv);
  a.io.tau_out = env_major(tau_out, nv);
  a.io.qdd_out = env_major(qdd_out, nv);
  a.integrate = integrate ? 1 : 0;
  a.dt = dt;
  a.q_state = const_cast<double*>(q);
  a.qd_state = const_cast<double*>(qd);
  auto s = static_cast<cudaStream_t>(stream);
  // models run with teams: the specialised one-warp-per-role sweep when it is available for
  // every one of them (run-time compilation on, sizes within its limits), each on a side
  // stream of the batch beside the persistent kernel, which takes the remaining tiles
  std::vector<int> roles;
  {
    bool ok = true;
    for (size_t m = 0; m < b->models.size() && ok; m++)
      if (b->lanes[m] > 1 && b->model_row_count[m] > 0) {
        std::string why;
        ok = step_roles_jit_ready(*b->models[m]->impl, b->lanes[m], ops, b->n, &why);
        roles.push_back(int(m));
      }
    if (!ok) roles.clear();
  }
  while (b->side.size() < roles.size()) {
    cudaStream_t st = nullptr;
    if (cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking) != cudaSuccess)
      return set_last_error(SGDYN_ERR_CUDA, "stream creation failed");
    b->side.push_back(st);
  }
  cudaError_t e = cudaSuccess;
  std::vector<cudaEvent_t> joins;
  cudaEvent_t fork = nullptr;
  if (!roles.empty()) {
    e = cudaEventCreateWithFlags(&fork, cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaEventRecord(fork, s);
    for (size_t r = 0; r < roles.size() && e == cudaSuccess; r++) {
      const int m = roles[r];
      e = cudaStreamWaitEvent(b->side[r], fork, 0);
      std::string why;
      if (e == cudaSuccess &&
          !launch_step_roles_rows_jit(*b->models[m]->impl, b->lanes[m], ops, a.io, b->model_rows + b->model_row_start[m],
                                      b->model_row_count[m], integrate ? dt : 0.0, integrate, b->side[r], &why))
        e = cudaErrorLaunchFailure;
      cudaEvent_t j = nullptr;
      if (e == cudaSuccess) e = cudaEventCreateWithFlags(&j, cudaEventDisableTiming);
      if (e == cudaSuccess) e = cudaEventRecord(j, b->side[r]);
      if (j) joins.push_back(j);
    }
    a.tiles = b->rest_tiles;
    a.ntiles = b->nrest;
  }
  if (e == cudaSuccess && a.ntiles > 0) {
    e = cudaMemsetAsync(b->head, 0, sizeof(unsigned int), s);
    dim3 grid(unsigned(b->sms * b->ctas_per_sm)), block(unsigned(32 * b->warps_per_cta));
    if (e == cudaSuccess)
      e = (b->max_nj <= 16) ? launch_hetero_bucket<16>(ops, a, grid, block, s)
                            : launch_hetero_bucket<32>(ops, a, grid, block, s);
  }
  for (cudaEvent_t j : joins) {
    if (e == cudaSuccess) e = cudaStreamWaitEvent(s, j, 0);
    cudaEventDestroy(j);  // released once the recorded work completes
  }
  if (fork) cudaEventDestroy(fork);
  if (e != cudaSuccess) return set_last_error(SGDYN_ERR_CUDA, std::string("kernel launch failed: ") + cudaGetErrorString(e));
  return SGDYN_OK;
}

int sgdyn_batch_step(sgdyn_batch* b, int ops, const double* q, const double* qd, const double* qdd, const double* tau,
                     double* link_poses, double* J, double* M, double* tau_out, double* qdd_out, void* stream) {
  SG_TRACE("sgdyn_batch_step");
  return batch_step(b, ops, q, qd, qdd, tau, link_poses, J, M, tau_out, qdd_out, stream, false, 0.0);
}

int sgdyn_batch_step_integrate(sgdyn_batch* b, double dt, double* q, double* qd, const double* tau, double* qdd_out,
                               void* stream) {
  SG_TRACE("sgdyn_batch_step_integrate");
  return batch_step(b, OP_ABA, q, qd, nullptr, tau, nullptr, nullptr, nullptr, nullptr, qdd_out, stream, true, dt);
}

}  // extern "C"
