// smat_internal.h — shared declarations of libsmat's host side.
#pragma once

#include <atomic>
#include <cstdint>
#include <mutex>
#include <string>
#include <vector>

#include "smat.h"
#include "spmm24.h"
#include "spmm_tc.h"

namespace smat {

// Thread-local last-error text behind smat_last_error().
void set_error(const std::string& msg);
smat_status fail(smat_status st, const std::string& msg);

// CUDA device ordinal a handle was built on (api.cu).
int bcsr_device(const smat_bcsr* A);

// A CUDA driver API function by name, looked up through the runtime
// (cudaGetDriverEntryPointByVersion), or nullptr. libsmat does not link
// libcuda, so that it loads (and its host-only entry points run) on machines
// without a GPU driver.
void* driver_fn(const char* name);

// ------------------------------------------------------------------ reorder
struct ReorderResult {
  std::vector<int64_t> grouping;
  std::vector<int64_t> perm;
  int64_t comparisons = 0;
  int64_t merges = 0;
};

// Distances of a chunk of Keeper candidates on a device: init() takes every
// row's block-column runs once; fill() writes, for rows j0 .. j1 - 1, the
// Jaccard distance (JaccardDistanceGroup, blocking.cpp:904-975) of the
// row's runs to the given pattern runs at group size g into out[j - j0]
// (every row, grouped or not: the caller reads the ones it compares).
struct KeeperDevice {
  virtual ~KeeperDevice() {}
  virtual bool init(const std::vector<int64_t>& runs, const std::vector<int64_t>& run_ptr) = 0;
  virtual bool fill(const int64_t* pattern, int64_t np, int64_t g, int64_t j0, int64_t j1, float* out) = 0;
  virtual const char* error() const = 0;
};
// A KeeperDevice on CUDA device `device` (reorder_gpu.cu); nullptr if the
// device cannot be used.
KeeperDevice* make_keeper_device(int device);

// Keeper grouping (blocking.cpp:431-547), bit-exact: the seed loop on the
// host; candidate distances on the host's cores, or on `dev` when given.
// Returns false when the device failed (its error() says why).
bool keeper_grouping(int64_t rows, const int64_t* rowptr, const int32_t* cols, float tau, int64_t col_block,
                     int64_t max_row_block, std::vector<int64_t>& grouping, int64_t& comparisons, int64_t& merges,
                     KeeperDevice* dev);
inline void keeper_grouping_host(int64_t rows, const int64_t* rowptr, const int32_t* cols, float tau,
                                 int64_t col_block, int64_t max_row_block, std::vector<int64_t>& grouping,
                                 int64_t& comparisons, int64_t& merges) {
  keeper_grouping(rows, rowptr, cols, tau, col_block, max_row_block, grouping, comparisons, merges, nullptr);
}
// get_permutation / get_fixed_size_grouping (utilities.cpp:8-20, 45-54).
std::vector<int64_t> permutation_of(const std::vector<int64_t>& grouping);
std::vector<int64_t> fixed_size_grouping(const std::vector<int64_t>& grouping, int64_t row_block);

// ------------------------------------------------------------------ BCSR
// Host-side BCSR structure (bh x bw blocks), bit-identical to csrToBcsr.
struct HostBcsr {
  int64_t rows = 0, cols = 0;        // logical
  int64_t rows_p = 0, cols_p = 0;    // padded
  int32_t bh = 16, bw = 16;
  int64_t nnz = 0;
  std::vector<int32_t> rowptr;       // nbr + 1
  std::vector<int32_t> colidx;       // nnzb, column start
  std::vector<float> val;            // nnzb * bh * bw (exact source values, FP32)
  std::vector<uint16_t> val_f16;     // same, as the FP16 the reference stores
  std::vector<int32_t> row_map;      // rows_p: BCSR row -> original row (or -1)
  std::vector<uint8_t> is24;         // per block: exactly 2:4 (values as FP16)
  std::vector<int32_t> kperm;        // permuted column -> original column (empty: none)
  int64_t nnzb() const { return (int64_t)colidx.size(); }
  int64_t nbr() const { return rows_p / bh; }
};

smat_status build_host_bcsr(const smat_csr& A, int32_t bh, int32_t bw, const int64_t* row_perm,
                            HostBcsr& out);

// HostBcsr from an existing BCSR (16 x 16 or 16 x 32 blocks, values FP16
// row-major per block, column starts), e.g. the arrays of the reference's
// SparseMatrix; 16 x 32 blocks are split into two 16 x 16 blocks.
smat_status build_host_bcsr_from_blocks(int64_t rows, int64_t cols, int32_t bh, int32_t bw, int64_t nnzb,
                                        const int32_t* row_ptr, const int32_t* col_idx, const uint16_t* vals,
                                        HostBcsr& out);

// Work plan of the tensor-core SpMM. Panels of `R` block rows; the blocks of
// a panel are ordered by block column (then block row) and cut into stages
// of at most stage_rows(cls) / bh blocks and stage_tiles(cls) block columns
// (cls: the plan class, spmm_tc.h). Each stage
// has a record (StageRec) and a header with its MMA list (spmm_tc.h).
struct Plan {
  int32_t R = 8;
  int32_t n_panels = 0;
  std::vector<PanelInfo> panels;
  std::vector<StageRec> stages;
  std::vector<int32_t> stream_blk;   // BCSR block index at each stream position
  std::vector<uint8_t> headers;      // stage headers, concatenated (StageRec::hdr_off)
  // C row of each plan row: inside a panel the block rows take TMEM slots in
  // an order that gives the MMA-issuing warps equal shares of the blocks
  std::vector<int32_t> row_map;
  int64_t n_groups = 0;              // MMA instructions per pass over A
  int64_t n_tiles = 0;               // B tile loads per pass over A
};

// skip (optional): blocks with skip[k] != 0 are left out of the plan (the
// exact-2:4 blocks that the structured-sparse path computes).
smat_status build_plan(const HostBcsr& b, int32_t R, int32_t cls, Plan& plan,
                       const std::vector<uint8_t>* skip = nullptr);

// ------------------------------------------------------------------ 2:4 path
// The structured-sparse path's units, stages and groups (spmm24.h) and the
// compressed stream, for the blocks with take[k] != 0 (16 x 16 blocks, all
// exactly 2:4); fmt 0: FP16 values, 1: BF16.
struct Sp24Host {
  std::vector<uint8_t> stream;
  std::vector<Sp24Stage> stages;
  std::vector<Sp24Group> groups;     // heaviest first
  std::vector<int32_t> unit_window;
  int64_t n_blocks = 0, n_units = 0;
};
smat_status build_sp24(const HostBcsr& b, const std::vector<uint8_t>& take, int fmt, Sp24Host& out);
// Blocks routed to the 2:4 path: exactly 2:4 (is24), in a unit (8 block
// rows x one 32-column window) holding at least min_unit such blocks.
void route_sp24(const HostBcsr& b, int min_unit, std::vector<uint8_t>& take);

// The reference's per-block sparsity label (csrToBcsr, matrix.h:679-711), per
// BCSR block: 1 = "2:4" (the default), 2 = dense once a row of the block has
// three consecutive columns (file order) ending at column % 4 in {2, 3}.
smat_status block_info_ref(const smat_csr& A, const int64_t* perm, const HostBcsr& b, std::vector<int8_t>& info);

// FP8 form: per block (BCSR order) the e4m3 codes of value / scale and one
// FP32 scale, chosen among candidates mapping the block's largest magnitude
// to 448 ... 224 to minimise the block's squared quantisation error.
smat_status quantize_fp8(const HostBcsr& b, std::vector<uint8_t>& q, std::vector<float>& scale);

// Work items of one launch shape: panels whose cost exceeds max_item_frac
// of the per-worker average are split into parts (stage ranges) of about
// that size. `order` lists the items by decreasing estimated cost: the CTAs
// of a launch take them in that order, each the next one when it is done
// with its last (the first from its own index). n_split = split panels,
// n_slabs = their parts (one partial-sum slab per part and column tile).
void build_work_items(const Plan& pl, int32_t bh, int32_t workers, double max_item_frac,
                      std::vector<WorkItem>& items, std::vector<int32_t>& order, int32_t& n_split,
                      int32_t& n_slabs);


// ------------------------------------------------------------------ handle
// Work list of one launch shape (NSUB).
struct Sched {
  int grid = 0;
  int32_t n_items = 0;
  int32_t* d_order = nullptr;  // items by decreasing estimated cost
  WorkItem* d_items = nullptr;
  int32_t n_split = 0;  // panels split into parts
  int32_t n_slabs = 0;  // parts of split panels
};

// A plan class's plan and its device copies and work lists.
struct PlanDev {
  Plan plan;
  bool built = false;
  PanelInfo* d_panels = nullptr;
  StageRec* d_stages = nullptr;
  int32_t* d_row_map = nullptr;
  Sched sched[3];  // by NSUB (1, 2)
};

struct SmatBcsrBody {
  int device = 0;
  HostBcsr host;
  int32_t R = 16;  // block rows per panel
  PlanDev pc[kPlanClasses];
  uint32_t forms = 0;
  int use24 = 0;
  int64_t n_24 = 0;
  // 2:4 path (use24 and 16 x 16 blocks): the groups, stages and unit windows
  // (shared by the forms) and one compressed stream per form (FP16, BF16)
  int sp24_on = 0;
  int32_t sp24_ngroups = 0;
  int64_t sp24_units = 0;
  Sp24Stage* d_sp24_stages = nullptr;
  Sp24Group* d_sp24_groups = nullptr;
  int32_t* d_sp24_unit_window = nullptr;
  uint8_t* d_sp24_stream[2] = {nullptr, nullptr};
  int32_t* d_bcsr_row_map = nullptr;  // [rows_padded] BCSR row -> C row
  int num_sms = 0;
  int32_t* d_kperm = nullptr;  // column permutation for the B gather (or null)
  // A stream per form (F16, BF16, -, SPLIT): per stage the pre-swizzled
  // blocks in consumption order (hi, then lo for the split form) and the
  // stage header
  uint8_t* d_aval[4] = {nullptr, nullptr, nullptr, nullptr};
  // the same for the 256-column plan (class 3): FP16, BF16
  uint8_t* d_aval_wide[2] = {nullptr, nullptr};
  int32_t depth = 0;                 // pipeline stages in flight (0: all that fit)
  // FP8 form, BCSR block order: e4m3 codes and per-block scales (for export)
  std::vector<uint8_t> fp8_q;
  std::vector<float> fp8_scale;
  int* d_err = nullptr;
  uint64_t wait_ns = 0;              // device-side wait limit (0: the kernels' default)
  std::atomic<int32_t> stall{0};     // testing hook: one-shot stall stage of the next launch
  // smat_spmm_host staging
  std::mutex mu;
  void* d_bstage = nullptr;
  size_t bstage_bytes = 0;
  void* d_cstage = nullptr;
  size_t cstage_bytes = 0;
  void* d_ws = nullptr;
  size_t ws_bytes = 0;
};


}  // namespace smat (the handle type is declared in the global namespace by smat.h)

struct smat_bcsr : smat::SmatBcsrBody {};

namespace smat {

// Kernel kind of an arithmetic form, its plan class, and the N-tile width
// (128 * nsub) used for N.
int kind_of(int32_t form);
inline int plan_class(int32_t form, int nsub = 1) {
  return form == SMAT_FORM_SPLIT_BF16 ? 1 : (form == SMAT_FORM_FP8 ? 2 : (nsub == 2 ? 3 : 0));
}
inline int plan_class_of_kind(int kind, int nsub = 1) {
  return kind == TC_KIND_SPLIT ? 1 : (kind == TC_KIND_FP8 ? 2 : (nsub == 2 ? 3 : 0));
}
// Block rows per panel when the caller leaves it to the library: 256 rows
// (16 blocks of 16 rows, 8 of 32), two TMEM accumulator buffers of 256
// columns; panels costing more than kDefaultSplitFrac of the average CTA
// load are split into parts.
inline int default_panel_rows(int bh) { return bh == 16 ? 16 : 8; }
constexpr double kDefaultSplitFrac = 0.5;
int pick_nsub(const smat_bcsr* h, int64_t N, int kind);

// Workspace layout of one SpMM: [packed B (x2 for the split form)]
// [the 2:4 path's copy of B, when the handle uses it for this form]
// [the launch's next-item counter, 16 bytes]
// [per split panel, column tile and TMEM lane quadrant: an int counter]
// [per part of a split panel and column tile: an R*bh x BN FP32 slab].
struct WsLayout {
  size_t counters = 0, counter_bytes = 0, slabs = 0, total = 0;
  size_t b64 = 0;  // the 2:4 path's copy of B (0: none)
};
WsLayout ws_layout(const smat_bcsr* A, int32_t form, int64_t N);

// The kernel's view of one SpMM: A's device plan and stream for the form,
// the packed B and scratch at `ws` (laid out as wl), C.
void fill_problem(const smat_bcsr* A, int32_t form, const void* ws, int64_t N, void* C, int32_t c_dtype,
                  int64_t ldc, int nsub, const WsLayout& wl, ProblemDesc& P);

// The same over several problems (WorkItem::prob = index into plans); the
// split decisions use the total over all problems; n_split / n_slabs per
// problem.
void build_work_items_multi(const std::vector<const Plan*>& plans, const std::vector<int32_t>& bhs, int32_t workers,
                            double max_item_frac, std::vector<WorkItem>& items, std::vector<int32_t>& order,
                            std::vector<int32_t>& n_split, std::vector<int32_t>& n_slabs);

// ------------------------------------------------------------------ autotuner
// Key of the tuning cache: block-density statistics of a matrix (blocks per
// block row and blocks per B tile of a 16-row panel, log2-bucketed), the
// N-tile count and the kernel kind.
struct TuneKey {
  int32_t bh = 16, bpr_bucket = 0, reuse_bucket = 0, ntile_bucket = 0, kind = 0;
  bool operator<(const TuneKey& o) const {
    if (bh != o.bh) return bh < o.bh;
    if (bpr_bucket != o.bpr_bucket) return bpr_bucket < o.bpr_bucket;
    if (reuse_bucket != o.reuse_bucket) return reuse_bucket < o.reuse_bucket;
    if (ntile_bucket != o.ntile_bucket) return ntile_bucket < o.ntile_bucket;
    return kind < o.kind;
  }
};
struct TuneVal {
  int32_t panel_rows = 16;
  float split_frac = 1.0f;
  int32_t n_tile_cols = 128;
  int32_t depth = 0;
  double ms = 0.0;
};
bool tune_key_of(const HostBcsr& b, int kind, int64_t N, TuneKey& key);
bool tune_lookup(const TuneKey& key, TuneVal& val);
void tune_store(const TuneKey& key, const TuneVal& val);

// Item indices by decreasing cost (ties by index).
void order_items(const std::vector<double>& item_cost, std::vector<int32_t>& order);

}  // namespace smat
