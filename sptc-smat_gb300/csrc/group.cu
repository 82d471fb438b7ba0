// group.cu — many SpMMs of uneven sizes in one persistent launch.
//
// smat_group_create takes a list of problems (handle, form, B, C, N) and
// builds, once, everything the launches need: one work list over all the
// problems' panels (heavy panels split into parts, longest-processing-time
// assignment to the CTAs, so that small and large problems share the GPU),
// the per-problem descriptors the kernel reads, the packed-B / partial-sum
// scratch and the jobs of the grouped B packing. smat_group_run then issues
// one grouped B-packing launch, one memset of the split-panel counters and
// one SpMM launch per kernel variant among the problems (one for a group of
// FP16 / BF16 problems with N <= 128), and allocates nothing, so it can be
// captured in a CUDA graph. The pointers B and C are fixed at creation.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>
#include <map>
#include <tuple>
#include <vector>

#include "convert.h"
#include "smat_internal.h"
#include "spmm_tc.h"

using namespace smat;

namespace {

struct Launch {
  int bh = 16, R = 16, nsub = 1, kind = 0, grid = 1;
  ProblemDesc* d_probs = nullptr;
  WorkItem* d_items = nullptr;
  int32_t* d_order = nullptr;
  int32_t n_items = 0;
  int32_t ctr = 0;  // int offset of the launch's next-item counter in d_counters
};

}  // namespace

struct smat_group {
  int device = 0;
  int num_sms = 0;
  uint8_t* d_ws = nullptr;       // packed B and partial sums of every problem
  int32_t* d_counters = nullptr;  // split-panel counters of every problem
  size_t counter_bytes = 0;
  PackJob* d_jobs = nullptr;
  int njobs = 0;
  int64_t pack_blocks = 0;
  int* d_err = nullptr;
  std::vector<Launch> launches;
};

static void group_free(smat_group* g) {
  if (!g) return;
  int prev = -1;
  cudaGetDevice(&prev);
  cudaSetDevice(g->device);
  for (Launch& l : g->launches) {
    cudaFree(l.d_probs);
    cudaFree(l.d_items);
    cudaFree(l.d_order);
  }
  cudaFree(g->d_ws);
  cudaFree(g->d_counters);
  cudaFree(g->d_jobs);
  cudaFree(g->d_err);
  if (prev >= 0) cudaSetDevice(prev);
  delete g;
}

template <typename T>
static cudaError_t upload_vec(T** d, const std::vector<T>& v) {
  *d = nullptr;
  cudaError_t e = cudaMalloc(reinterpret_cast<void**>(d), std::max<size_t>(v.size(), 1) * sizeof(T));
  if (e == cudaSuccess && !v.empty()) e = cudaMemcpy(*d, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice);
  return e;
}

extern "C" {

smat_status smat_group_create(const smat_problem* probs, int32_t count, smat_group** out) {
  if (!probs || !out || count < 0) return fail(SMAT_ERR_INVALID, "null argument");
  *out = nullptr;
  if (count == 0) return fail(SMAT_ERR_INVALID, "empty group");
  if (!probs[0].A) return fail(SMAT_ERR_INVALID, "problem 0: null handle");
  const int device = bcsr_device(probs[0].A);
  // validate, and sort the problems into kernel variants
  std::map<std::tuple<int, int, int, int>, std::vector<int32_t>> variants;
  for (int32_t i = 0; i < count; i++) {
    const smat_problem& p = probs[i];
    if (!p.A || !p.B || !p.C) return fail(SMAT_ERR_INVALID, "problem " + std::to_string(i) + ": null pointer");
    if (bcsr_device(p.A) != device) return fail(SMAT_ERR_INVALID, "all problems of a group must be on one device");
    if (p.form < 0 || p.form > 3 || !(p.A->forms & (1u << p.form)))
      return fail(SMAT_ERR_INVALID, "problem " + std::to_string(i) + ": form was not materialised");
    if (p.N <= 0 || p.N > (1 << 30)) return fail(SMAT_ERR_INVALID, "problem " + std::to_string(i) + ": bad N");
    if (p.b_dtype != SMAT_F32 && p.b_dtype != SMAT_F16 && p.b_dtype != SMAT_BF16)
      return fail(SMAT_ERR_INVALID, "B must be F32, F16 or BF16");
    if (p.b_layout != SMAT_ROW_MAJOR && p.b_layout != SMAT_COL_MAJOR) return fail(SMAT_ERR_INVALID, "bad B layout");
    if (p.b_layout == SMAT_COL_MAJOR ? p.ldb < p.A->host.cols : p.ldb < p.N) return fail(SMAT_ERR_INVALID, "ldb too small");
    if (p.c_dtype != SMAT_F32 && p.c_dtype != SMAT_F16) return fail(SMAT_ERR_INVALID, "C must be F32 or F16");
    if (p.ldc < p.N) return fail(SMAT_ERR_INVALID, "ldc < N");
    const int kind = kind_of(p.form);
    const int nsub = pick_nsub(p.A, p.N, kind);
    if (!tc_variant_supported(p.A->host.bh, p.A->R, nsub, kind))
      return fail(SMAT_ERR_UNSUPPORTED, "problem " + std::to_string(i) + ": no kernel variant");
    variants[{p.A->host.bh, p.A->R, nsub, kind}].push_back(i);
  }
  int prev = -1;
  cudaGetDevice(&prev);
  if (cudaSetDevice(device) != cudaSuccess) return fail(SMAT_ERR_CUDA, "cudaSetDevice failed");
  struct Restore {
    int prev, dev;
    ~Restore() {
      if (prev >= 0 && prev != dev) cudaSetDevice(prev);
    }
  } restore{prev, device};
  smat_group* g = new smat_group();
  g->device = device;
  cudaDeviceGetAttribute(&g->num_sms, cudaDevAttrMultiProcessorCount, device);
#define GTRY(x)                                          \
  do {                                                   \
    cudaError_t e_ = (x);                                \
    if (e_ != cudaSuccess) {                             \
      group_free(g);                                     \
      return fail(SMAT_ERR_CUDA, std::string(#x ": ") + cudaGetErrorString(e_)); \
    }                                                    \
  } while (0)

  // work lists per variant; per problem its scratch sizes
  struct Scratch {
    size_t packed = 0, slabs = 0, ws_off = 0, ctr_off = 0, ctr_n = 0;
  };
  std::vector<Scratch> sc(count);
  std::vector<std::vector<WorkItem>> v_items;
  std::vector<std::vector<int32_t>> v_order;
  std::vector<std::vector<int32_t>> v_members;
  for (auto& kv : variants) {
    const auto& members = kv.second;
    const int bh = std::get<0>(kv.first), nsub = std::get<2>(kv.first), kind = std::get<3>(kv.first);
    std::vector<const Plan*> plans;
    std::vector<int32_t> bhs;
    for (int32_t i : members) {
      plans.push_back(&probs[i].A->pc[plan_class_of_kind(kind, nsub)].plan);
      bhs.push_back(probs[i].A->host.bh);
    }
    const int workers = std::max(1, g->num_sms * tc_ctas_per_sm(bh, std::get<1>(kv.first), nsub, kind));
    std::vector<WorkItem> items;
    std::vector<int32_t> order, n_split, n_slabs;
    build_work_items_multi(plans, bhs, workers, 1.0, items, order, n_split, n_slabs);
    for (size_t m = 0; m < members.size(); m++) {
      const smat_problem& p = probs[members[m]];
      const int64_t bn = 128 * nsub, n_tiles = (p.N + bn - 1) / bn;
      Scratch& s = sc[members[m]];
      const size_t one = (packed_b_bytes(p.A->host.cols, p.N) + 255) / 256 * 256;
      s.packed = kind == TC_KIND_SPLIT ? 2 * one : one;
      s.slabs = (size_t)n_slabs[m] * n_tiles * p.A->R * p.A->host.bh * bn * sizeof(float);
      s.ctr_n = (size_t)n_split[m] * n_tiles * 4;
    }
    Launch l;
    l.bh = bh;
    l.R = std::get<1>(kv.first);
    l.nsub = nsub;
    l.kind = kind;
    l.grid = std::max(1, std::min<int>(workers, (int)items.size()));
    l.n_items = (int32_t)items.size();
    g->launches.push_back(l);
    v_items.push_back(std::move(items));
    v_order.push_back(std::move(order));
    v_members.push_back(members);
  }
  // one scratch allocation for all problems, one for all counters: each
  // launch's next-item counter (16 bytes apart), then the split panels'
  size_t ws_total = 0, ctr_total = 4 * g->launches.size();
  for (size_t v = 0; v < g->launches.size(); v++) g->launches[v].ctr = (int32_t)(4 * v);
  for (Scratch& s : sc) {
    s.ws_off = ws_total;
    ws_total += (s.packed + s.slabs + 255) / 256 * 256;
    s.ctr_off = ctr_total;
    ctr_total += s.ctr_n;
  }
  GTRY(cudaMalloc(reinterpret_cast<void**>(&g->d_ws), std::max<size_t>(ws_total, 256)));
  g->counter_bytes = ctr_total * sizeof(int32_t);
  GTRY(cudaMalloc(reinterpret_cast<void**>(&g->d_counters), std::max<size_t>(g->counter_bytes, 256)));
  GTRY(cudaMalloc(reinterpret_cast<void**>(&g->d_err), sizeof(int)));
  GTRY(cudaMemset(g->d_err, 0, sizeof(int)));
  // descriptors and pack jobs
  std::vector<PackJob> jobs(count);
  int64_t blocks = 0;
  for (int32_t i = 0; i < count; i++) {
    const smat_problem& p = probs[i];
    PackJob& j = jobs[i];
    j.in = p.B;
    j.out = g->d_ws + sc[i].ws_off;
    j.kperm = p.A->d_kperm;
    j.ldi = p.ldb;
    j.K = p.A->host.cols;
    j.N = p.N;
    j.begin = blocks;
    j.in_dtype = p.b_dtype == SMAT_F32 ? 0 : (p.b_dtype == SMAT_F16 ? 1 : 2);
    j.layout = p.b_layout == SMAT_COL_MAJOR ? 1 : 0;
    j.out_mode = (p.form == SMAT_FORM_F16 || p.form == SMAT_FORM_FP8) ? 0 : (p.form == SMAT_FORM_SPLIT_BF16 ? 2 : 1);
    j.ntiles = (int32_t)packed_b_tiles(p.N);
    blocks += (int64_t)j.ntiles * ((p.A->host.cols + 15) / 16);
  }
  g->njobs = count;
  g->pack_blocks = blocks;
  GTRY(upload_vec(&g->d_jobs, jobs));
  for (size_t v = 0; v < g->launches.size(); v++) {
    Launch& l = g->launches[v];
    std::vector<ProblemDesc> descs(v_members[v].size());
    for (size_t m = 0; m < v_members[v].size(); m++) {
      const int32_t i = v_members[v][m];
      const smat_problem& p = probs[i];
      WsLayout wl;  // offsets are replaced below
      fill_problem(p.A, p.form, g->d_ws + sc[i].ws_off, p.N, p.C, p.c_dtype, p.ldc, l.nsub, wl, descs[m]);
      descs[m].slabs = reinterpret_cast<float*>(g->d_ws + sc[i].ws_off + sc[i].packed);
      descs[m].counters = g->d_counters + sc[i].ctr_off;
    }
    GTRY(upload_vec(&l.d_probs, descs));
    GTRY(upload_vec(&l.d_items, v_items[v]));
    GTRY(upload_vec(&l.d_order, v_order[v]));
  }
#undef GTRY
  *out = g;
  return SMAT_OK;
}

smat_status smat_group_run(smat_group* g, void* stream_) {
  if (!g) return fail(SMAT_ERR_INVALID, "null group");
  int prev = -1;
  cudaGetDevice(&prev);
  if (prev != g->device && cudaSetDevice(g->device) != cudaSuccess) return fail(SMAT_ERR_CUDA, "cudaSetDevice failed");
  const cudaStream_t s = static_cast<cudaStream_t>(stream_);
  smat_status st = SMAT_OK;
  cudaError_t e = pack_b_grouped(g->d_jobs, g->njobs, g->pack_blocks, g->num_sms, s);
  if (e != cudaSuccess) st = fail(SMAT_ERR_CUDA, std::string("grouped B packing: ") + cudaGetErrorString(e));
  if (st == SMAT_OK && g->counter_bytes) {
    e = cudaMemsetAsync(g->d_counters, 0, g->counter_bytes, s);
    if (e != cudaSuccess) st = fail(SMAT_ERR_CUDA, "clearing the split-panel counters");
  }
  for (size_t v = 0; v < g->launches.size() && st == SMAT_OK; v++) {
    const Launch& l = g->launches[v];
    SpmmArgs args;
    std::memset(&args, 0, sizeof(args));
    args.probs = l.d_probs;
    args.order = l.d_order;
    args.n_items = l.n_items;
    args.next_item = g->d_counters + l.ctr;
    args.items = l.d_items;
    args.err = g->d_err;
    e = tc_launch(l.bh, l.R, l.nsub, l.kind, args, l.grid, s);
    if (e != cudaSuccess) st = fail(SMAT_ERR_CUDA, std::string("grouped spmm launch: ") + cudaGetErrorString(e));
  }
  if (prev >= 0 && prev != g->device) cudaSetDevice(prev);
  return st;
}

smat_status smat_group_check_device_error(smat_group* g) {
  if (!g) return fail(SMAT_ERR_INVALID, "null group");
  int v = 0;
  if (cudaMemcpy(&v, g->d_err, sizeof(int), cudaMemcpyDeviceToHost) != cudaSuccess)
    return fail(SMAT_ERR_CUDA, "reading the group's error word");
  if (v != 0) {
    const int zero = 0;
    cudaMemcpy(g->d_err, &zero, sizeof(int), cudaMemcpyHostToDevice);
    return fail(SMAT_ERR_TIMEOUT, "device-side wait timed out at site " + std::to_string(v));
  }
  return SMAT_OK;
}

smat_status smat_group_destroy(smat_group* g) {
  group_free(g);
  return SMAT_OK;
}

}  // extern "C"
