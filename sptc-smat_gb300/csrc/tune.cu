// tune.cu — the SpMM autotuner.
//
// smat_autotune measures the launch shapes the library offers for a matrix
// on the device, with CUDA events: block rows per panel R (the rows one CTA
// work item covers), how far heavy panels are split across CTAs, the N-tile
// width (128 columns per pass over A, or 256 when N > 128 and R <= 8, where
// the two accumulator buffers still fit tensor memory) and then, for the best
// of those, the pipeline depth (stages in flight). It keeps the fastest in a
// process-wide cache keyed on the matrix's block-density statistics: blocks
// per block row and blocks per B tile inside a 16-row panel (how much one B
// tile is reused), both log2-bucketed, plus the N-tile count and the kernel
// kind.
// smat_bcsr_create with panel_rows = 0 looks its matrix up in that cache, so
// one tuning run serves every matrix with similar statistics.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <map>
#include <mutex>
#include <vector>

#include "smat_internal.h"
#include "spmm_tc.h"

namespace smat {
namespace {
std::mutex g_tune_mu;
std::map<TuneKey, TuneVal> g_tune;
}  // namespace

bool tune_key_of(const HostBcsr& b, int kind, int64_t N, TuneKey& key) {
  const int64_t nbr = b.nbr(), nnzb = b.nnzb();
  if (nbr == 0 || nnzb == 0) return false;
  // blocks per B tile over 16-row panels (distinct block columns per panel)
  int64_t distinct = 0;
  std::vector<int32_t> stamp((b.cols_p + b.bw - 1) / b.bw + 1, -1);
  for (int64_t p0 = 0; p0 < nbr; p0 += 16) {
    for (int64_t br = p0; br < std::min(nbr, p0 + 16); br++)
      for (int32_t k = b.rowptr[br]; k < b.rowptr[br + 1]; k++) {
        const int32_t c = b.colidx[k] / b.bw;
        if (stamp[c] != (int32_t)p0) {
          stamp[c] = (int32_t)p0;
          distinct++;
        }
      }
  }
  key.bh = b.bh;
  key.bpr_bucket = (int32_t)std::lround(2.0 * std::log2(1.0 + (double)nnzb / nbr));
  key.reuse_bucket = (int32_t)std::lround(4.0 * std::log2((double)nnzb / std::max<int64_t>(1, distinct)));
  key.ntile_bucket = (int32_t)std::min<int64_t>(8, (std::max<int64_t>(N, 1) + 127) / 128);
  key.kind = kind;
  return true;
}

bool tune_lookup(const TuneKey& key, TuneVal& val) {
  std::lock_guard<std::mutex> lock(g_tune_mu);
  auto it = g_tune.find(key);
  if (it == g_tune.end()) return false;
  val = it->second;
  return true;
}

void tune_store(const TuneKey& key, const TuneVal& val) {
  std::lock_guard<std::mutex> lock(g_tune_mu);
  g_tune[key] = val;
}

}  // namespace smat

using namespace smat;

extern "C" {

smat_status smat_autotune(const smat_csr* A, const smat_bcsr_opts* opts, int32_t form, int64_t N,
                          smat_tune_result* out) {
  if (!A || !out) return fail(SMAT_ERR_INVALID, "null argument");
  if (form < 0 || form > 3 || N <= 0) return fail(SMAT_ERR_INVALID, "bad form or N");
  smat_bcsr_opts o{};
  if (opts) o = *opts;
  const int bh = o.block_rows ? o.block_rows : 16;
  const int bw = o.block_cols ? o.block_cols : 16;
  HostBcsr hb;
  smat_status st = build_host_bcsr(*A, bh, bw, o.row_perm, hb);
  if (st != SMAT_OK) return st;
  TuneKey key;
  if (!tune_key_of(hb, kind_of(form), N, key)) return fail(SMAT_ERR_INVALID, "empty matrix: nothing to tune");
  std::memset(out, 0, sizeof(*out));
  TuneVal cached;
  if (tune_lookup(key, cached)) {
    out->panel_rows = cached.panel_rows;
    out->split_frac = cached.split_frac;
    out->n_tile_cols = cached.n_tile_cols;
    out->pipeline_depth = cached.depth;
    out->ms = cached.ms;
    out->cached = 1;
    return SMAT_OK;
  }
  const std::vector<int> Rs = bh == 16 ? std::vector<int>{4, 8, 16} : std::vector<int>{4, 8};
  const std::vector<float> fracs = {-1.0f, 2.0f, 1.0f, 0.5f};
  int prev = -1;
  cudaGetDevice(&prev);
  if (cudaSetDevice(o.device) != cudaSuccess) return fail(SMAT_ERR_CUDA, "cudaSetDevice failed");
  // operands: FP32 B (every form packs from it), FP32 C, the largest workspace
  const int64_t K = hb.cols, M = hb.rows;
  void *dB = nullptr, *dC = nullptr, *dW = nullptr;
  size_t wbytes = 0;
  cudaStream_t s = nullptr;
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  bool ok = cudaMalloc(&dB, (size_t)std::max<int64_t>(K, 1) * N * 4) == cudaSuccess &&
            cudaMalloc(&dC, (size_t)std::max<int64_t>(M, 1) * N * 4) == cudaSuccess &&
            cudaMemset(dB, 0x3c, (size_t)std::max<int64_t>(K, 1) * N * 4) == cudaSuccess &&
            cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking) == cudaSuccess &&
            cudaEventCreate(&e0) == cudaSuccess && cudaEventCreate(&e1) == cudaSuccess;
  TuneVal best;
  best.ms = INFINITY;
  double ms_default = 0.0;
  int candidates = 0;
  // one candidate: build the handle, 3 warm-up and 8 timed SpMMs; < 0 when
  // the shape is not offered for this form, NaN on a failure
  auto measure = [&](int R, float f, int ntc, int depth) -> double {
    smat_bcsr_opts oc = o;
    oc.panel_rows = R;
    oc.split_frac = f;
    oc.n_tile_cols = ntc;
    oc.pipeline_depth = depth;
    oc.forms = 1u << form;
    smat_bcsr* h = nullptr;
    if (smat_bcsr_create(A, &oc, &h) != SMAT_OK) return -1.0;  // shape not offered for this form
    size_t need = 0;
    smat_spmm_workspace_size(h, form, SMAT_F32, N, &need);
    if (need > wbytes) {
      cudaFree(dW);
      dW = nullptr;
      wbytes = 0;
      if (cudaMalloc(&dW, need) != cudaSuccess) {
        smat_bcsr_destroy(h);
        return NAN;
      }
      wbytes = need;
    }
    float ms = 0.0f;
    bool run_ok = true;
    for (int i = 0; i < 3 && run_ok; i++)
      run_ok = smat_spmm(h, form, dB, SMAT_F32, SMAT_ROW_MAJOR, N, dC, SMAT_F32, N, N, dW, wbytes, s) == SMAT_OK;
    constexpr int kReps = 8;
    run_ok = run_ok && cudaEventRecord(e0, s) == cudaSuccess;
    for (int i = 0; i < kReps && run_ok; i++)
      run_ok = smat_spmm(h, form, dB, SMAT_F32, SMAT_ROW_MAJOR, N, dC, SMAT_F32, N, N, dW, wbytes, s) == SMAT_OK;
    run_ok = run_ok && cudaEventRecord(e1, s) == cudaSuccess && cudaEventSynchronize(e1) == cudaSuccess &&
             cudaEventElapsedTime(&ms, e0, e1) == cudaSuccess && smat_bcsr_check_device_error(h) == SMAT_OK;
    smat_bcsr_destroy(h);
    if (!run_ok) return NAN;
    candidates++;
    return ms / kReps;
  };
  auto consider = [&](double t, int R, float f, int ntc, int depth) {
    if (t >= 0.0 && t < best.ms) {
      best.ms = t;
      best.panel_rows = R;
      best.split_frac = f;
      best.n_tile_cols = ntc;
      best.depth = depth;
    }
  };
  // panel height x splitting threshold x N-tile width
  for (int R : Rs) {
    for (float f : fracs) {
      for (int ntc : {128, 256}) {
        if (!ok) break;
        if (ntc == 256 && (N <= 128 || !tc_variant_supported(bh, R, 2, kind_of(form)))) continue;
        const double t = measure(R, f, ntc, 0);
        if (std::isnan(t)) {
          ok = false;
          break;
        }
        if (R == default_panel_rows(bh) && f == (float)kDefaultSplitFrac && ntc == 128) ms_default = t;
        consider(t, R, f, ntc, 0);
      }
    }
  }
  // pipeline depth of the best shape: 0 (every stage slot that fits in
  // shared memory: 3 for every stage shape offered) against 2
  if (ok && std::isfinite(best.ms)) {
    const TuneVal b0 = best;
    for (int depth : {2}) {
      const double t = measure(b0.panel_rows, b0.split_frac, b0.n_tile_cols, depth);
      if (std::isnan(t)) {
        ok = false;
        break;
      }
      consider(t, b0.panel_rows, b0.split_frac, b0.n_tile_cols, depth);
    }
  }
  cudaFree(dB);
  cudaFree(dC);
  cudaFree(dW);
  if (e0) cudaEventDestroy(e0);
  if (e1) cudaEventDestroy(e1);
  if (s) cudaStreamDestroy(s);
  if (prev >= 0) cudaSetDevice(prev);
  if (!ok || !std::isfinite(best.ms)) return fail(SMAT_ERR_CUDA, "autotuning failed: " + std::string(smat_last_error()));
  tune_store(key, best);
  out->panel_rows = best.panel_rows;
  out->split_frac = best.split_frac;
  out->n_tile_cols = best.n_tile_cols;
  out->pipeline_depth = best.depth;
  out->ms = best.ms;
  out->ms_default = ms_default;
  out->cached = 0;
  out->candidates = candidates;
  return SMAT_OK;
}

smat_status smat_autotune_clear(void) {
  std::lock_guard<std::mutex> lock(g_tune_mu);
  g_tune.clear();
  return SMAT_OK;
}

}  // extern "C"
