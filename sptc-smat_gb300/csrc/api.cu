// api.cu — the C ABI declared in include/smat.h.
#include <cuda.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <memory>
#include <mutex>
#include <string>
#include <vector>

#include "convert.h"
#include "fp_convert.h"
#include "smat_internal.h"
#include "spmm_tc.h"

namespace smat {

static thread_local std::string g_last_error;

void set_error(const std::string& msg) { g_last_error = msg; }
smat_status fail(smat_status st, const std::string& msg) {
  g_last_error = msg;
  return st;
}

void* driver_fn(const char* name) {
  void* fn = nullptr;
  cudaDriverEntryPointQueryResult q = cudaDriverEntryPointSymbolNotFound;
  if (cudaGetDriverEntryPointByVersion(name, &fn, 12000, cudaEnableDefault, &q) != cudaSuccess ||
      q != cudaDriverEntryPointSuccess) {
    cudaGetLastError();
    return nullptr;
  }
  return fn;
}

static smat_status cuda_fail(cudaError_t e, const char* what) {
  return fail(SMAT_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
}

#define SMAT_CUDA(call)                               \
  do {                                                \
    cudaError_t e_ = (call);                          \
    if (e_ != cudaSuccess) return cuda_fail(e_, #call); \
  } while (0)

// RAII: make `dev` current, restore the caller's device afterwards.
struct DeviceGuard {
  int prev = -1;
  bool ok = true;
  explicit DeviceGuard(int dev) {
    if (cudaGetDevice(&prev) != cudaSuccess) prev = -1;
    if (prev != dev) ok = cudaSetDevice(dev) == cudaSuccess;
  }
  ~DeviceGuard() {
    int cur = -1;
    if (prev >= 0 && cudaGetDevice(&cur) == cudaSuccess && cur != prev) cudaSetDevice(prev);
  }
};

template <typename T>
static smat_status upload(T** dptr, const T* src, size_t n) {
  *dptr = nullptr;
  size_t bytes = std::max<size_t>(n, 1) * sizeof(T);
  SMAT_CUDA(cudaMalloc(reinterpret_cast<void**>(dptr), bytes));
  if (n) SMAT_CUDA(cudaMemcpy(*dptr, src, n * sizeof(T), cudaMemcpyHostToDevice));
  return SMAT_OK;
}

}  // namespace smat

using namespace smat;

static void free_handle(smat_bcsr* h) {
  if (!h) return;
  int prev = -1;
  cudaGetDevice(&prev);
  cudaSetDevice(h->device);
  void* ptrs[] = {h->d_kperm, h->d_aval[0], h->d_aval[1], h->d_aval[2], h->d_aval[3], h->d_err,
                  h->d_bstage, h->d_cstage, h->d_ws, h->d_sp24_stages, h->d_sp24_groups,
                  h->d_sp24_unit_window, h->d_sp24_stream[0], h->d_sp24_stream[1], h->d_bcsr_row_map,
                  h->d_aval_wide[0], h->d_aval_wide[1]};
  for (void* p : ptrs)
    if (p) cudaFree(p);
  for (PlanDev& pd : h->pc) {
    void* pp[] = {pd.d_stages, pd.d_panels, pd.d_row_map, pd.sched[1].d_order, pd.sched[1].d_items,
                  pd.sched[2].d_order, pd.sched[2].d_items};
    for (void* p : pp)
      if (p) cudaFree(p);
  }
  if (prev >= 0) cudaSetDevice(prev);
  delete h;
}

// Kernel kind of an arithmetic form.
int smat::kind_of(int32_t form) {
  return form == SMAT_FORM_SPLIT_BF16 ? TC_KIND_SPLIT : (form == SMAT_FORM_FP8 ? TC_KIND_FP8 : TC_KIND_PLAIN);
}

int smat::pick_nsub(const smat_bcsr* h, int64_t N, int kind) {
  // 256-column passes where the handle holds their plan (opts.n_tile_cols)
  if (N > 128 && kind == TC_KIND_PLAIN && h->pc[3].built && tc_variant_supported(h->host.bh, h->R, 2, kind))
    return 2;
  return 1;
}

int smat::bcsr_device(const smat_bcsr* A) { return A->device; }

// Second half of handle creation, shared by the CSR and BCSR entry points:
// the work plan, the device copies and the schedules. Frees h on failure.
static smat_status finish_handle(smat_bcsr* h, const smat_bcsr_opts& o, smat_bcsr** out) {
  const int bh = h->host.bh, bw = h->host.bw;
  const uint32_t forms = h->forms;
  smat_status st;
  // heavy panels are split over CTAs below
  int R = o.panel_rows ? o.panel_rows : default_panel_rows(bh);
  float split_frac = o.split_frac;
  int ntc = o.n_tile_cols, depth = o.pipeline_depth;
  if (o.panel_rows == 0) {
    // a configuration the autotuner measured for matrices like this one
    // (measured for N <= 128 first, else for N <= 256)
    for (int64_t n_try : {128, 256}) {
      TuneKey key;
      TuneVal tv;
      if (tune_key_of(h->host, kind_of(SMAT_FORM_F16), n_try, key) && tune_lookup(key, tv)) {
        R = tv.panel_rows;
        if (o.split_frac == 0.0f) split_frac = tv.split_frac;
        if (o.n_tile_cols == 0) ntc = tv.n_tile_cols;
        if (o.pipeline_depth == 0) depth = tv.depth;
        break;
      }
    }
  }
  if ((ntc != 0 && ntc != 128 && ntc != 256) || depth < 0 || depth == 1) {
    delete h;
    return fail(SMAT_ERR_INVALID, "n_tile_cols must be 0, 128 or 256 and pipeline_depth 0 or >= 2");
  }
  h->depth = depth;
  if (!tc_variant_supported(bh, R, 1, TC_KIND_PLAIN)) {
    delete h;
    return fail(SMAT_ERR_UNSUPPORTED, "unsupported panel_rows for this block height");
  }
  h->R = R;
  // class 0 serves the FP16 and BF16 forms (and the handle's info), class 1
  // the split form, class 2 the FP8 form
  // the structured-sparse path takes the exact-2:4 blocks of the FP16 and
  // BF16 forms (16 x 16 blocks); their plan (class 0) leaves them out
  // (use_24 = the fewest such blocks a unit -- 8 block rows x 32 columns --
  // must hold for its blocks to be routed there)
  std::vector<uint8_t> take24;
  if (h->use24 > 0 && bh == 16 && bw == 16 && (forms & ((1u << SMAT_FORM_F16) | (1u << SMAT_FORM_BF16))))
    route_sp24(h->host, h->use24, take24);
  h->sp24_on = std::any_of(take24.begin(), take24.end(), [](uint8_t v) { return v != 0; });
  const bool wide = ntc == 256 && (forms & ((1u << SMAT_FORM_F16) | (1u << SMAT_FORM_BF16))) &&
                    tc_variant_supported(bh, R, 2, TC_KIND_PLAIN);
  for (int cls = 0; cls < kPlanClasses; cls++) {
    if (cls == 1 && !(forms & (1u << SMAT_FORM_SPLIT_BF16))) continue;
    if (cls == 2 && !(forms & (1u << SMAT_FORM_FP8))) continue;
    if (cls == 3 && !wide) continue;
    st = build_plan(h->host, R, cls, h->pc[cls].plan, ((cls == 0 || cls == 3) && h->sp24_on) ? &take24 : nullptr);
    if (st != SMAT_OK) {
      delete h;
      return st;
    }
    h->pc[cls].built = true;
  }
  if (h->sp24_on)
    for (uint8_t v : take24) h->n_24 += v;

#define SMAT_TRY(x)              \
  do {                           \
    smat_status s_ = (x);        \
    if (s_ != SMAT_OK) {         \
      free_handle(h);            \
      return s_;                 \
    }                            \
  } while (0)

  const HostBcsr& b = h->host;
  if (!b.kperm.empty()) SMAT_TRY(upload(&h->d_kperm, b.kperm.data(), b.kperm.size()));
  if (h->sp24_on) {
    Sp24Host sp;
    for (int fmt = 0; fmt < 2; fmt++) {
      if (!(forms & (1u << (fmt == 0 ? SMAT_FORM_F16 : SMAT_FORM_BF16)))) continue;
      SMAT_TRY(build_sp24(b, take24, fmt, sp));
      SMAT_TRY(upload(&h->d_sp24_stream[fmt], sp.stream.data(), sp.stream.size()));
    }
    // (some block is routed to the 2:4 path, so every list below has an entry)
    SMAT_TRY(upload(&h->d_sp24_stages, sp.stages.data(), sp.stages.size()));
    SMAT_TRY(upload(&h->d_sp24_groups, sp.groups.data(), sp.groups.size()));
    SMAT_TRY(upload(&h->d_sp24_unit_window, sp.unit_window.data(), sp.unit_window.size()));
    SMAT_TRY(upload(&h->d_bcsr_row_map, b.row_map.data(), b.row_map.size()));
    h->sp24_ngroups = (int32_t)sp.groups.size();
    h->sp24_units = sp.n_units;
  }
  {
    int zero = 0;
    SMAT_TRY(upload(&h->d_err, &zero, 1));
  }
  const double frac = split_frac == 0.0f ? kDefaultSplitFrac : (split_frac < 0.0f ? 1e30 : (double)split_frac);
  for (int cls = 0; cls < kPlanClasses; cls++) {
    PlanDev& pd = h->pc[cls];
    if (!pd.built) continue;
    SMAT_TRY(upload(&pd.d_stages, pd.plan.stages.data(), pd.plan.stages.size()));
    SMAT_TRY(upload(&pd.d_panels, pd.plan.panels.data(), pd.plan.panels.size()));
    SMAT_TRY(upload(&pd.d_row_map, pd.plan.row_map.data(), pd.plan.row_map.size()));
    // work items per launch shape (NSUB 1 and 2): heavy panels split into
    // parts so that no CTA gets much more than the average
    const int kind = cls == 1 ? TC_KIND_SPLIT : (cls == 2 ? TC_KIND_FP8 : TC_KIND_PLAIN);
    for (int nsub = 1; nsub <= 2; nsub++) {
      if (plan_class_of_kind(kind, nsub) != cls || !tc_variant_supported(bh, R, nsub, kind)) continue;
      const int per_sm = tc_ctas_per_sm(bh, R, nsub, kind);
      const int workers = std::max(1, h->num_sms * per_sm);
      std::vector<WorkItem> items;
      std::vector<int32_t> order;
      Sched& sc = pd.sched[nsub];
      build_work_items(pd.plan, bh, workers, frac, items, order, sc.n_split, sc.n_slabs);
      sc.grid = std::max(1, std::min<int>(workers, (int)items.size()));
      sc.n_items = (int32_t)items.size();
      SMAT_TRY(upload(&sc.d_items, items.data(), items.size()));
      SMAT_TRY(upload(&sc.d_order, order.data(), order.size()));
    }
  }

  // A streams, one per requested form: for each stage its blocks in
  // consumption order in the 32-byte-swizzled shared-memory layout (inside
  // each 256-byte group of 8 rows of 32 bytes, the two 16-byte halves of
  // rows 4..7 are swapped), hi then lo blocks for the split form, then the
  // stage header.
  const int64_t nnzb = b.nnzb();
  const size_t bsz = (size_t)bh * bw, ablk = (size_t)bh * 32;
  auto stream_layout = [&](const Plan& pl, const std::vector<uint16_t>& hi, const std::vector<uint16_t>* lo,
                           std::vector<uint8_t>& out) {
    const int64_t nst = (int64_t)pl.stages.size();
    const size_t nops = lo ? 2 : 1;
    out.assign(std::max<size_t>((size_t)nnzb * ablk * nops + pl.headers.size(), 16), 0);
    auto put = [&](const std::vector<uint16_t>& vals, int64_t k, uint8_t* dst) {
      const uint8_t* src = reinterpret_cast<const uint8_t*>(vals.data() + (size_t)pl.stream_blk[k] * bsz);
      for (int r = 0; r < bh; r++)
        for (int c = 0; c < 2; c++)
          std::memcpy(dst + r * 32 + ((c ^ ((r >> 2) & 1)) * 16), src + r * 32 + c * 16, 16);
    };
#pragma omp parallel for schedule(static)
    for (int64_t si = 0; si < nst; si++) {
      const StageRec& r = pl.stages[si];
      uint8_t* base = out.data() + (size_t)r.blk_off * ablk * nops + (size_t)r.hdr_off;
      for (int32_t q = 0; q < r.nblk; q++) {
        put(hi, r.blk_off + q, base + (size_t)q * ablk);
        if (lo) put(*lo, r.blk_off + q, base + ((size_t)r.nblk + q) * ablk);
      }
      std::memcpy(base + (size_t)r.nblk * ablk * nops, pl.headers.data() + r.hdr_off, (size_t)r.hdr_bytes);
    }
  };
  std::vector<uint8_t> lay;
  const size_t nval = (size_t)nnzb * bsz;
  if (forms & (1u << SMAT_FORM_F16)) {
    stream_layout(h->pc[0].plan, b.val_f16, nullptr, lay);
    SMAT_TRY(upload(&h->d_aval[SMAT_FORM_F16], lay.data(), lay.size()));
    if (wide) {
      stream_layout(h->pc[3].plan, b.val_f16, nullptr, lay);
      SMAT_TRY(upload(&h->d_aval_wide[0], lay.data(), lay.size()));
    }
  }
  if (forms & ((1u << SMAT_FORM_BF16) | (1u << SMAT_FORM_SPLIT_BF16))) {
    std::vector<uint16_t> hi(nval), lo(nval);
    for (size_t i = 0; i < nval; i++) {
      hi[i] = f32_to_bf16_bits(b.val[i]);
      lo[i] = f32_to_bf16_bits(b.val[i] - bf16_bits_to_f32(hi[i]));
    }
    if (forms & (1u << SMAT_FORM_BF16)) {
      stream_layout(h->pc[0].plan, hi, nullptr, lay);
      SMAT_TRY(upload(&h->d_aval[SMAT_FORM_BF16], lay.data(), lay.size()));
      if (wide) {
        stream_layout(h->pc[3].plan, hi, nullptr, lay);
        SMAT_TRY(upload(&h->d_aval_wide[1], lay.data(), lay.size()));
      }
    }
    if (forms & (1u << SMAT_FORM_SPLIT_BF16)) {
      stream_layout(h->pc[1].plan, hi, &lo, lay);
      SMAT_TRY(upload(&h->d_aval[SMAT_FORM_SPLIT_BF16], lay.data(), lay.size()));
    }
  }
  if (forms & (1u << SMAT_FORM_FP8)) {
    if (bh != 16) {
      free_handle(h);
      return fail(SMAT_ERR_UNSUPPORTED, "FP8 form: 16 x 16 blocks only");
    }
    SMAT_TRY(quantize_fp8(b, h->fp8_q, h->fp8_scale));
    const Plan& pl = h->pc[2].plan;
    const int64_t nst = (int64_t)pl.stages.size();
    // per stage: [nblk e4m3 blocks][nblk FP32 scales, padded][header]
    lay.assign(std::max<size_t>((size_t)nnzb * 256 + pl.headers.size() +
                                    (nst ? (size_t)pl.stages[nst - 1].scl_off + fp8_scale_bytes(pl.stages[nst - 1].nblk) : 0),
                                16),
               0);
#pragma omp parallel for schedule(static)
    for (int64_t si = 0; si < nst; si++) {
      const StageRec& r = pl.stages[si];
      uint8_t* base = lay.data() + (size_t)r.blk_off * 256 + (size_t)r.scl_off + (size_t)r.hdr_off;
      for (int32_t qb = 0; qb < r.nblk; qb++) {
        const int64_t blk = pl.stream_blk[r.blk_off + qb];
        std::memcpy(base + (size_t)qb * 256, h->fp8_q.data() + (size_t)blk * 256, 256);
        std::memcpy(base + (size_t)r.nblk * 256 + (size_t)qb * 4, &h->fp8_scale[blk], 4);
      }
      std::memcpy(base + (size_t)r.nblk * 256 + fp8_scale_bytes(r.nblk), pl.headers.data() + r.hdr_off,
                  (size_t)r.hdr_bytes);
    }
    SMAT_TRY(upload(&h->d_aval[SMAT_FORM_FP8], lay.data(), lay.size()));
  }
  // keep the FP16 values for export; the FP32 copy is no longer needed
  std::vector<float>().swap(h->host.val);
#undef SMAT_TRY
  *out = h;
  return SMAT_OK;
}

extern "C" {

const char* smat_last_error(void) { return g_last_error.c_str(); }
const char* smat_version(void) { return "smat-gb300 0.1 (sm_103a, tcgen05)"; }

smat_status smat_reorder(const smat_csr* A, float tau, int32_t col_block, int32_t row_block,
                         int32_t algo, int32_t force_fixed, int32_t use_gpu, int64_t* perm_out,
                         int64_t* grouping_out, smat_reorder_stats* stats) {
  if (!A || !perm_out) return fail(SMAT_ERR_INVALID, "null argument");
  if (A->rows < 0 || !A->row_ptr || (A->nnz > 0 && !A->col_idx))
    return fail(SMAT_ERR_INVALID, "malformed CSR");
  if (col_block < 1 || row_block < 1) return fail(SMAT_ERR_INVALID, "block sizes must be >= 1");
  if (A->row_ptr[0] != 0 || A->row_ptr[A->rows] != A->nnz)
    return fail(SMAT_ERR_INVALID, "row_ptr[0] must be 0 and row_ptr[rows] == nnz");
  for (int64_t r = 0; r < A->rows; r++)
    if (A->row_ptr[r + 1] < A->row_ptr[r]) return fail(SMAT_ERR_INVALID, "row_ptr not monotone");
  for (int64_t k = 0; k < A->nnz; k++)
    if (A->col_idx[k] < 0) return fail(SMAT_ERR_INVALID, "negative column index");
  std::vector<int64_t> g;
  int64_t comparisons = 0, merges = 0;
  if (algo == 5) {
    if (use_gpu) {
      // candidate distances on the current CUDA device, commit on the host
      int d = 0;
      if (cudaGetDevice(&d) != cudaSuccess) return fail(SMAT_ERR_NO_DEVICE, "use_gpu: no CUDA device");
      std::unique_ptr<KeeperDevice> kd(make_keeper_device(d));
      if (!kd) return fail(SMAT_ERR_NO_DEVICE, "use_gpu: no CUDA device");
      if (!keeper_grouping(A->rows, A->row_ptr, A->col_idx, tau, col_block, row_block, g, comparisons, merges,
                           kd.get()))
        return fail(SMAT_ERR_CUDA, std::string("use_gpu: ") + kd->error());
    } else {
      keeper_grouping_host(A->rows, A->row_ptr, A->col_idx, tau, col_block, row_block, g, comparisons, merges);
    }
  } else if (algo == 2) {
    // FixedBlocking (blocking.cpp:551-559)
    g.resize(A->rows);
    for (int64_t i = 0; i < A->rows; i++) g[i] = i / row_block;
  } else {
    return fail(SMAT_ERR_UNSUPPORTED, "only algorithms 5 (Keeper) and 2 (fixed) are implemented");
  }
  if (force_fixed && algo != 2) g = fixed_size_grouping(g, row_block);
  std::vector<int64_t> p = permutation_of(g);
  std::copy(p.begin(), p.end(), perm_out);
  if (grouping_out) std::copy(g.begin(), g.end(), grouping_out);
  if (stats) {
    stats->comparisons = comparisons;
    stats->merges = merges;
  }
  return SMAT_OK;
}

// Checks the device and allocates the handle shell.
static smat_status new_handle(const smat_bcsr_opts& o, uint32_t forms, smat_bcsr** hp) {
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0)
    return fail(SMAT_ERR_NO_DEVICE, "no CUDA device");
  if (o.device < 0 || o.device >= ndev) return fail(SMAT_ERR_INVALID, "bad device ordinal");
  DeviceGuard guard(o.device);
  if (!guard.ok) return fail(SMAT_ERR_CUDA, "cudaSetDevice failed");
  cudaDeviceProp prop;
  SMAT_CUDA(cudaGetDeviceProperties(&prop, o.device));
  if (prop.major != 10 || prop.minor != 3)
    return fail(SMAT_ERR_NO_DEVICE, "libsmat kernels are built for sm_103a (GB300) only");
  smat_bcsr* h = new smat_bcsr();
  h->device = o.device;
  h->forms = forms;
  h->use24 = o.use_24;
  h->num_sms = prop.multiProcessorCount;
  *hp = h;
  return SMAT_OK;
}

smat_status smat_bcsr_create(const smat_csr* A, const smat_bcsr_opts* opts, smat_bcsr** out) {
  if (!A || !out) return fail(SMAT_ERR_INVALID, "null argument");
  *out = nullptr;
  smat_bcsr_opts o{};
  if (opts) o = *opts;
  const int bh = o.block_rows ? o.block_rows : 16;
  const int bw = o.block_cols ? o.block_cols : 16;
  if (bw != 16 || (bh != 16 && bh != 32))
    return fail(SMAT_ERR_UNSUPPORTED, "tensor-core path supports 16x16 and 32x16 blocks");
  const uint32_t forms = o.forms ? o.forms : (1u << SMAT_FORM_F16);
  smat_bcsr* h = nullptr;
  smat_status st = new_handle(o, forms, &h);
  if (st != SMAT_OK) return st;
  DeviceGuard guard(o.device);
  if (o.col_perm) {
    // block the matrix with its columns permuted: new column inv[old]
    std::vector<int32_t> inv(std::max<int64_t>(A->cols, 0), -1);
    for (int64_t c = 0; c < A->cols; c++) {
      const int64_t src = o.col_perm[c];
      if (src < 0 || src >= A->cols || inv[src] >= 0) {
        delete h;
        return fail(SMAT_ERR_INVALID, "col_perm is not a permutation");
      }
      inv[src] = (int32_t)c;
    }
    std::vector<int32_t> ci(std::max<int64_t>(A->nnz, 0));
    for (int64_t k = 0; k < A->nnz; k++) {
      const int32_t c = A->col_idx[k];
      if (c < 0 || c >= A->cols) {
        delete h;
        return fail(SMAT_ERR_INVALID, "column index out of range");
      }
      ci[k] = inv[c];
    }
    smat_csr A2 = *A;
    A2.col_idx = ci.data();
    st = build_host_bcsr(A2, bh, bw, o.row_perm, h->host);
    h->host.kperm.assign(o.col_perm, o.col_perm + A->cols);
  } else {
    st = build_host_bcsr(*A, bh, bw, o.row_perm, h->host);
  }
  if (st != SMAT_OK) {
    delete h;
    return st;
  }
  return finish_handle(h, o, out);
}

smat_status smat_bcsr_create_from_bcsr(int64_t rows, int64_t cols, int32_t block_rows, int32_t block_cols,
                                       int64_t nnzb, const int32_t* row_ptr, const int32_t* col_idx,
                                       const uint16_t* values_f16, const smat_bcsr_opts* opts, smat_bcsr** out) {
  if (!out) return fail(SMAT_ERR_INVALID, "null argument");
  *out = nullptr;
  smat_bcsr_opts o{};
  if (opts) o = *opts;
  if (o.row_perm) return fail(SMAT_ERR_UNSUPPORTED, "row_perm applies to CSR input only");
  const uint32_t forms = o.forms ? o.forms : (1u << SMAT_FORM_F16);
  smat_bcsr* h = nullptr;
  smat_status st = new_handle(o, forms, &h);
  if (st != SMAT_OK) return st;
  DeviceGuard guard(o.device);
  st = build_host_bcsr_from_blocks(rows, cols, block_rows, block_cols, nnzb, row_ptr, col_idx, values_f16, h->host);
  if (st != SMAT_OK) {
    delete h;
    return st;
  }
  return finish_handle(h, o, out);
}

smat_status smat_bcsr_destroy(smat_bcsr* A) {
  free_handle(A);
  return SMAT_OK;
}

smat_status smat_bcsr_export_fp8(const smat_bcsr* A, uint8_t* codes, float* scales) {
  if (!A) return fail(SMAT_ERR_INVALID, "null handle");
  if (!(A->forms & (1u << SMAT_FORM_FP8))) return fail(SMAT_ERR_INVALID, "FP8 form was not materialised");
  if (codes) std::copy(A->fp8_q.begin(), A->fp8_q.end(), codes);
  if (scales) std::copy(A->fp8_scale.begin(), A->fp8_scale.end(), scales);
  return SMAT_OK;
}

smat_status smat_bcsr_get_info(const smat_bcsr* A, smat_bcsr_info* info) {
  if (!A || !info) return fail(SMAT_ERR_INVALID, "null argument");
  const HostBcsr& b = A->host;
  info->rows = b.rows;
  info->cols = b.cols;
  info->rows_padded = b.rows_p;
  info->cols_padded = b.cols_p;
  info->nnz = b.nnz;
  info->nnzb = b.nnzb();
  info->n_blocks_24 = A->n_24;
  info->block_rows = b.bh;
  info->block_cols = b.bw;
  info->panel_rows = A->R;
  info->n_panels = A->pc[0].plan.n_panels;
  {
    int64_t u = 0;
    for (const auto& p : A->pc[0].plan.panels) u += p.nucol;
    info->n_union_cols = u;
  }
  info->fill = b.nnzb() ? (double)b.nnz / ((double)b.nnzb() * b.bh * b.bw) : 0.0;
  info->n_tile_cols = A->pc[3].built ? 256 : 128;
  info->pipeline_depth = A->depth;
  return SMAT_OK;
}

smat_status smat_bcsr_export(const smat_bcsr* A, int32_t* row_ptr, int32_t* col_idx,
                             uint16_t* values_f16, uint8_t* is_24) {
  if (!A) return fail(SMAT_ERR_INVALID, "null argument");
  const HostBcsr& b = A->host;
  if (row_ptr) std::copy(b.rowptr.begin(), b.rowptr.end(), row_ptr);
  if (col_idx) std::copy(b.colidx.begin(), b.colidx.end(), col_idx);
  if (values_f16) std::copy(b.val_f16.begin(), b.val_f16.end(), values_f16);
  if (is_24) std::copy(b.is24.begin(), b.is24.end(), is_24);
  return SMAT_OK;
}

smat_status smat_csr_to_bcsr_host(const smat_csr* A, int32_t block_rows, int32_t block_cols,
                                  const int64_t* row_perm, int64_t* nnzb, int32_t* row_ptr,
                                  int32_t* col_idx, uint16_t* values_f16) {
  if (!A || !nnzb) return fail(SMAT_ERR_INVALID, "null argument");
  HostBcsr b;
  smat_status st = build_host_bcsr(*A, block_rows ? block_rows : 16, block_cols ? block_cols : 16,
                                   row_perm, b);
  if (st != SMAT_OK) return st;
  *nnzb = b.nnzb();
  if (row_ptr) std::copy(b.rowptr.begin(), b.rowptr.end(), row_ptr);
  if (col_idx) std::copy(b.colidx.begin(), b.colidx.end(), col_idx);
  if (values_f16) std::copy(b.val_f16.begin(), b.val_f16.end(), values_f16);
  return SMAT_OK;
}

}  // extern "C"

// The 2:4 path runs for this form (the exact-2:4 blocks are not in its plan).
static bool uses_sp24(const smat_bcsr* A, int32_t form) {
  return A->sp24_on && (form == SMAT_FORM_F16 || form == SMAT_FORM_BF16);
}

WsLayout smat::ws_layout(const smat_bcsr* A, int32_t form, int64_t N) {
  WsLayout w;
  const bool split = form == SMAT_FORM_SPLIT_BF16;
  const size_t one = (packed_b_bytes(A->host.cols, std::max<int64_t>(N, 1)) + 255) / 256 * 256;
  w.counters = split ? 2 * one : one;
  if (uses_sp24(A, form)) {
    w.b64 = w.counters;
    w.counters += (packed_b64_bytes(A->host.cols, std::max<int64_t>(N, 1)) + 255) / 256 * 256;
  }
  const int nsub = pick_nsub(A, N, kind_of(form));
  const Sched& sc = A->pc[plan_class(form, nsub)].sched[nsub];
  const int64_t bn = 128 * nsub, n_tiles = (std::max<int64_t>(N, 1) + bn - 1) / bn;
  w.counter_bytes = (16 + (size_t)sc.n_split * n_tiles * 4 * sizeof(int32_t) + 255) / 256 * 256;
  w.slabs = w.counters + w.counter_bytes;
  w.total = w.slabs + (size_t)sc.n_slabs * n_tiles * A->R * A->host.bh * bn * sizeof(float);
  return w;
}

// The kernel's view of one SpMM: A's device plan and stream for the form,
// the packed B and scratch at `ws` (laid out as ws_layout), C.
void smat::fill_problem(const smat_bcsr* A, int32_t form, const void* ws_, int64_t N, void* C, int32_t c_dtype,
                        int64_t ldc, int nsub, const WsLayout& wl, ProblemDesc& P) {
  std::memset(&P, 0, sizeof(P));
  uint8_t* ws = const_cast<uint8_t*>(static_cast<const uint8_t*>(ws_));
  const int64_t bn = 128 * nsub;
  P.bpack = ws;
  P.bp_kbs = (A->host.cols + 15) / 16;
  const int cls = plan_class(form, nsub);
  P.aval = cls == 3 ? A->d_aval_wide[form == SMAT_FORM_BF16 ? 1 : 0] : A->d_aval[form];
  P.panels = A->pc[cls].d_panels;
  P.stages = A->pc[cls].d_stages;
  P.row_map = A->pc[cls].d_row_map;
  P.C = C;
  P.ldc = ldc;
  P.counters = reinterpret_cast<int32_t*>(ws + wl.counters + 16);  // after the next-item counter
  P.slabs = reinterpret_cast<float*>(ws + wl.slabs);
  P.N = (int32_t)N;
  P.n_tiles = (int32_t)((N + bn - 1) / bn);
  P.nbr = A->pc[cls].plan.n_panels * A->pc[cls].plan.R;  // plan rows (slots)
  P.c_f16 = c_dtype == SMAT_F16;
  // instruction descriptor (kind::f16): FP32 accumulator, FP16 (0) or BF16 (1)
  // operands, both K-major, M = 128; the kernel adds N per MMA group
  const uint32_t fmt = (form == SMAT_FORM_F16 || form == SMAT_FORM_FP8) ? 0u : 1u;
  P.idesc = (1u << 4) | (fmt << 7) | (fmt << 10) | ((uint32_t)(128 >> 4) << 24);
}

extern "C" {

smat_status smat_csr_to_bcsr_split_host(const smat_csr* A, int32_t block_cols, const int64_t* row_perm,
                                        int64_t* n_24, int64_t* n_dense, int32_t* row_ptr_24, int32_t* col_idx_24,
                                        uint16_t* values_24, int32_t* row_ptr_dense, int32_t* col_idx_dense,
                                        uint16_t* values_dense, int32_t* block_info) {
  if (!A || !n_24 || !n_dense) return fail(SMAT_ERR_INVALID, "null argument");
  HostBcsr b;
  smat_status st = build_host_bcsr(*A, 16, block_cols, row_perm, b);
  if (st != SMAT_OK) return st;
  std::vector<int8_t> info;
  block_info_ref(*A, row_perm, b, info);
  const int64_t nbr = b.nbr(), nbc = b.cols_p / b.bw, bsz = 16 * (int64_t)b.bw;
  int64_t c24 = 0, cd = 0;
  for (int8_t v : info) (v == 1 ? c24 : cd)++;
  *n_24 = c24;
  *n_dense = cd;
  if (block_info) {
    std::fill(block_info, block_info + nbr * nbc, 0);
    for (int64_t br = 0; br < nbr; br++)
      for (int32_t k = b.rowptr[br]; k < b.rowptr[br + 1]; k++) block_info[br * nbc + b.colidx[k] / b.bw] = info[k];
  }
  if (!row_ptr_24) return SMAT_OK;
  int64_t i24 = 0, id = 0;
  row_ptr_24[0] = 0;
  if (row_ptr_dense) row_ptr_dense[0] = 0;
  for (int64_t br = 0; br < nbr; br++) {
    for (int32_t k = b.rowptr[br]; k < b.rowptr[br + 1]; k++) {
      if (info[k] == 1) {
        if (col_idx_24) col_idx_24[i24] = b.colidx[k];
        if (values_24) std::copy(b.val_f16.begin() + k * bsz, b.val_f16.begin() + (k + 1) * bsz, values_24 + i24 * bsz);
        i24++;
      } else {
        if (col_idx_dense) col_idx_dense[id] = b.colidx[k];
        if (values_dense)
          std::copy(b.val_f16.begin() + k * bsz, b.val_f16.begin() + (k + 1) * bsz, values_dense + id * bsz);
        id++;
      }
    }
    row_ptr_24[br + 1] = (int32_t)i24;
    if (row_ptr_dense) row_ptr_dense[br + 1] = (int32_t)id;
  }
  return SMAT_OK;
}

smat_status smat_spmm_workspace_size(const smat_bcsr* A, int32_t form, int32_t b_dtype, int64_t N,
                                     size_t* bytes) {
  if (!A || !bytes) return fail(SMAT_ERR_INVALID, "null argument");
  (void)b_dtype;
  *bytes = ws_layout(A, form, N).total;
  return SMAT_OK;
}

static smat_status check_common(const smat_bcsr* A, int32_t form, int64_t N) {
  if (!A) return fail(SMAT_ERR_INVALID, "null handle");
  if (form < 0 || form > 3 || !(A->forms & (1u << form)))
    return fail(SMAT_ERR_INVALID, "form was not materialised when the handle was built");
  if (N <= 0 || N > (1 << 30)) return fail(SMAT_ERR_INVALID, "bad N");
  return SMAT_OK;
}

smat_status smat_spmm_pack_b(const smat_bcsr* A, int32_t form, const void* B, int32_t b_dtype,
                             int32_t b_layout, int64_t ldb, int64_t N, void* workspace,
                             size_t workspace_bytes, void* stream_) {
  smat_status st = check_common(A, form, N);
  if (st != SMAT_OK) return st;
  if (!B) return fail(SMAT_ERR_INVALID, "null B");
  if (b_layout != SMAT_ROW_MAJOR && b_layout != SMAT_COL_MAJOR) return fail(SMAT_ERR_INVALID, "bad B layout");
  if (b_dtype != SMAT_F32 && b_dtype != SMAT_F16 && b_dtype != SMAT_BF16)
    return fail(SMAT_ERR_INVALID, "B must be F32, F16 or BF16");
  const int64_t K = A->host.cols;
  if (b_layout == SMAT_COL_MAJOR ? ldb < K : ldb < N) return fail(SMAT_ERR_INVALID, "ldb too small");
  size_t need = 0;
  smat_spmm_workspace_size(A, form, b_dtype, N, &need);
  if (!workspace || workspace_bytes < need)
    return fail(SMAT_ERR_INVALID, "workspace too small (see smat_spmm_workspace_size)");
  if (reinterpret_cast<uintptr_t>(workspace) & 255) return fail(SMAT_ERR_INVALID, "workspace must be 256-byte aligned");
  DeviceGuard guard(A->device);
  if (!guard.ok) return fail(SMAT_ERR_CUDA, "cudaSetDevice failed");
  const bool split = form == SMAT_FORM_SPLIT_BF16;
  uint8_t* out = static_cast<uint8_t*>(workspace);
  const int in_dt = b_dtype == SMAT_F32 ? 0 : (b_dtype == SMAT_F16 ? 1 : 2);
  const int mode = (form == SMAT_FORM_F16 || form == SMAT_FORM_FP8) ? 0 : (split ? 2 : 1);
  cudaError_t e = pack_b(B, in_dt, b_layout == SMAT_COL_MAJOR ? 1 : 0, ldb, mode, out, K, N, A->d_kperm,
                         static_cast<cudaStream_t>(stream_));
  if (e != cudaSuccess) return cuda_fail(e, "pack_b");
  if (uses_sp24(A, form)) {
    const WsLayout wl = ws_layout(A, form, N);
    e = pack_b_sw64(out, K, N, out + wl.b64, static_cast<cudaStream_t>(stream_));
    if (e != cudaSuccess) return cuda_fail(e, "pack_b_sw64");
  }
  return SMAT_OK;
}

smat_status smat_spmm_packed(const smat_bcsr* A, int32_t form, const void* packed_b, int64_t N,
                             void* C, int32_t c_dtype, int64_t ldc, void* stream_) {
  smat_status st = check_common(A, form, N);
  if (st != SMAT_OK) return st;
  if (!packed_b || !C) return fail(SMAT_ERR_INVALID, "null argument");
  if (c_dtype != SMAT_F32 && c_dtype != SMAT_F16) return fail(SMAT_ERR_INVALID, "C must be F32 or F16");
  if (ldc < N) return fail(SMAT_ERR_INVALID, "ldc < N");
  const HostBcsr& hb = A->host;
  if (hb.rows == 0) return SMAT_OK;
  DeviceGuard guard(A->device);
  if (!guard.ok) return fail(SMAT_ERR_CUDA, "cudaSetDevice failed");
  const int kind = kind_of(form);
  const int nsub = pick_nsub(A, N, kind);
  const int bh = hb.bh, R = A->R;
  if (!tc_variant_supported(bh, R, nsub, kind)) return fail(SMAT_ERR_UNSUPPORTED, "no kernel variant");
  const Sched& sc = A->pc[plan_class(form, nsub)].sched[nsub];
  SpmmArgs args;
  std::memset(&args, 0, sizeof(args));
  const WsLayout wl = ws_layout(A, form, N);
  fill_problem(A, form, packed_b, N, C, c_dtype, ldc, nsub, wl, args.one);
  args.order = sc.d_order;
  args.n_items = sc.n_items;
  args.items = sc.d_items;
  args.err = A->d_err;
  args.wait_ns = A->wait_ns;
  args.stall_stage = const_cast<smat_bcsr*>(A)->stall.exchange(0);
  args.depth = A->depth;
  uint8_t* ctr = static_cast<uint8_t*>(const_cast<void*>(packed_b)) + wl.counters;
  args.next_item = reinterpret_cast<int32_t*>(ctr);
  {
    // the next-item counter and the split panels' counters start at zero
    // in every launch
    cudaError_t e = cudaMemsetAsync(ctr, 0, wl.counter_bytes, static_cast<cudaStream_t>(stream_));
    if (e != cudaSuccess) return cuda_fail(e, "clearing the work counters");
  }
  cudaError_t e = tc_launch(bh, R, nsub, kind, args, sc.grid, static_cast<cudaStream_t>(stream_));
  if (e != cudaSuccess) return cuda_fail(e, "spmm kernel launch");
  if (uses_sp24(A, form)) {
    // the exact-2:4 blocks, added into the C the dense kernel wrote
    Sp24Args a24;
    std::memset(&a24, 0, sizeof(a24));
    const int fmt = form == SMAT_FORM_BF16 ? 1 : 0;
    a24.stream = A->d_sp24_stream[fmt];
    a24.stages = A->d_sp24_stages;
    a24.groups = A->d_sp24_groups;
    a24.unit_window = A->d_sp24_unit_window;
    a24.row_map = A->d_bcsr_row_map;
    a24.bpack64 = static_cast<const uint8_t*>(packed_b) + wl.b64;
    a24.kw = ((hb.cols + 15) / 16 + 1) / 2;
    a24.C = C;
    a24.ldc = ldc;
    a24.N = (int32_t)N;
    a24.n_tiles = (int32_t)((N + 127) / 128);
    a24.n_groups = A->sp24_ngroups;
    a24.c_f16 = c_dtype == SMAT_F16 ? 1 : 0;
    // kind::f16 instruction descriptor without N: sparse (bit 2), FP32
    // accumulator, A and B FP16 (0) or BF16 (1), K-major, M = 128
    a24.idesc = (1u << 2) | (1u << 4) | ((uint32_t)fmt << 7) | ((uint32_t)fmt << 10) | ((uint32_t)(128 >> 4) << 24);
    a24.err = A->d_err;
    a24.wait_ns = A->wait_ns;
    const int grid = std::max(1, std::min<int>(A->num_sms, A->sp24_ngroups));
    e = sp24_launch(a24, grid, static_cast<cudaStream_t>(stream_));
    if (e != cudaSuccess) return cuda_fail(e, "2:4 spmm kernel launch");
  }
  return SMAT_OK;
}

smat_status smat_spmm(const smat_bcsr* A, int32_t form, const void* B, int32_t b_dtype,
                      int32_t b_layout, int64_t ldb, void* C, int32_t c_dtype, int64_t ldc,
                      int64_t N, void* workspace, size_t workspace_bytes, void* stream) {
  if (!A || !B || !C) return fail(SMAT_ERR_INVALID, "null argument");
  if (c_dtype != SMAT_F32 && c_dtype != SMAT_F16) return fail(SMAT_ERR_INVALID, "C must be F32 or F16");
  if (ldc < N) return fail(SMAT_ERR_INVALID, "ldc < N");
  smat_status st = smat_spmm_pack_b(A, form, B, b_dtype, b_layout, ldb, N, workspace, workspace_bytes, stream);
  if (st != SMAT_OK) return st;
  return smat_spmm_packed(A, form, workspace, N, C, c_dtype, ldc, stream);
}

smat_status smat_spmm_host(const smat_bcsr* A_, int32_t form, const void* B_host, int32_t b_dtype,
                           int32_t b_layout, int64_t ldb, void* C_host, int32_t c_dtype,
                           int64_t ldc, int64_t N, void* stream_) {
  if (!A_ || !B_host || !C_host) return fail(SMAT_ERR_INVALID, "null argument");
  smat_bcsr* A = const_cast<smat_bcsr*>(A_);
  std::lock_guard<std::mutex> lock(A->mu);
  cudaStream_t stream = static_cast<cudaStream_t>(stream_);
  DeviceGuard guard(A->device);
  const int64_t K = A->host.cols, M = A->host.rows;
  const size_t belt = b_dtype == SMAT_F32 ? 4 : 2, celt = c_dtype == SMAT_F16 ? 2 : 4;
  const size_t bbytes = (b_layout == SMAT_COL_MAJOR) ? (size_t)ldb * (N - 1) * belt + K * belt
                                                     : (size_t)ldb * (K - 1) * belt + N * belt;
  const size_t cbytes = (size_t)ldc * (M - 1) * celt + N * celt;
  size_t wbytes = 0;
  smat_spmm_workspace_size(A, form, b_dtype, N, &wbytes);
  auto grow = [](void** p, size_t* cap, size_t need) -> cudaError_t {
    if (*cap >= need) return cudaSuccess;
    if (*p) cudaFree(*p);
    *p = nullptr;
    *cap = 0;
    cudaError_t e = cudaMalloc(p, need);
    if (e == cudaSuccess) *cap = need;
    return e;
  };
  SMAT_CUDA(grow(&A->d_ws, &A->ws_bytes, wbytes));
  // On GB300 the GPU reaches page-locked host memory directly over
  // NVLink-C2C: when both buffers are pinned, B is read and C written in
  // place by the pack and SpMM kernels, and no staging copies are made.
  cudaPointerAttributes pa{}, pc{};
  const bool b_pinned = cudaPointerGetAttributes(&pa, B_host) == cudaSuccess && pa.type == cudaMemoryTypeHost &&
                        pa.devicePointer != nullptr;
  const bool c_pinned = cudaPointerGetAttributes(&pc, C_host) == cudaSuccess && pc.type == cudaMemoryTypeHost &&
                        pc.devicePointer != nullptr;
  cudaGetLastError();
  if (b_pinned && c_pinned) {
    smat_status s = smat_spmm(A, form, pa.devicePointer, b_dtype, b_layout, ldb, pc.devicePointer, c_dtype, ldc, N,
                              A->d_ws, A->ws_bytes, stream);
    if (s != SMAT_OK) return s;
    SMAT_CUDA(cudaStreamSynchronize(stream));
    return SMAT_OK;
  }
  SMAT_CUDA(grow(&A->d_bstage, &A->bstage_bytes, bbytes));
  SMAT_CUDA(grow(&A->d_cstage, &A->cstage_bytes, std::max<size_t>(cbytes, 1)));
  SMAT_CUDA(cudaMemcpyAsync(A->d_bstage, B_host, bbytes, cudaMemcpyHostToDevice, stream));
  smat_status s = smat_spmm(A, form, A->d_bstage, b_dtype, b_layout, ldb, A->d_cstage, c_dtype, ldc,
                            N, A->d_ws, A->ws_bytes, stream);
  if (s != SMAT_OK) return s;
  SMAT_CUDA(cudaMemcpyAsync(C_host, A->d_cstage, cbytes, cudaMemcpyDeviceToHost, stream));
  SMAT_CUDA(cudaStreamSynchronize(stream));
  return SMAT_OK;
}

smat_status smat_bcsr_set_wait_limit(smat_bcsr* A, uint64_t ns) {
  if (!A) return fail(SMAT_ERR_INVALID, "null argument");
  A->wait_ns = ns;
  return SMAT_OK;
}

smat_status smat_bcsr_debug_stall(smat_bcsr* A, int32_t stage) {
  if (!A) return fail(SMAT_ERR_INVALID, "null argument");
  if (stage < 0) return fail(SMAT_ERR_INVALID, "stage must be >= 0");
  A->stall.store(stage);
  return SMAT_OK;
}

smat_status smat_bcsr_check_device_error(const smat_bcsr* A) {
  if (!A) return fail(SMAT_ERR_INVALID, "null argument");
  DeviceGuard guard(A->device);
  int v = 0;
  SMAT_CUDA(cudaMemcpy(&v, A->d_err, sizeof(int), cudaMemcpyDeviceToHost));
  if (v != 0) {
    int zero = 0;
    cudaMemcpy(A->d_err, &zero, sizeof(int), cudaMemcpyHostToDevice);
    return fail(SMAT_ERR_TIMEOUT, "device-side wait timed out at site " + std::to_string(v));
  }
  return SMAT_OK;
}

}  // extern "C"
