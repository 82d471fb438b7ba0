// smat_internal.h — shared declarations of libsmat's host side.
#pragma once

#include <cstdint>
#include <string>
#include <vector>

#include "smat.h"
#include "spmm_tc.h"

namespace smat {

// Thread-local last-error text behind smat_last_error().
void set_error(const std::string& msg);
smat_status fail(smat_status st, const std::string& msg);

// CUDA device ordinal a handle was built on (api.cu).
int bcsr_device(const smat_bcsr* A);

// ------------------------------------------------------------------ reorder
struct ReorderResult {
  std::vector<int64_t> grouping;
  std::vector<int64_t> perm;
  int64_t comparisons = 0;
  int64_t merges = 0;
};

// Keeper grouping (blocking.cpp:431-547) on the host, bit-exact.
void keeper_grouping_host(int64_t rows, const int64_t* rowptr, const int32_t* cols, float tau,
                          int64_t col_block, int64_t max_row_block, std::vector<int64_t>& grouping,
                          int64_t& comparisons, int64_t& merges);
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
// of at most kStageRows / bh blocks and kStageTiles block columns. Each stage
// has a record (StageRec) and a header with its MMA list (spmm_tc.h).
struct Plan {
  int32_t R = 8;
  int32_t n_panels = 0;
  std::vector<PanelInfo> panels;
  std::vector<StageRec> stages;
  std::vector<int32_t> stream_blk;   // BCSR block index at each stream position
  std::vector<uint8_t> headers;      // stage headers, concatenated (StageRec::hdr_off)
  int64_t n_groups = 0;              // MMA instructions per pass over A
  int64_t n_tiles = 0;               // B tile loads per pass over A
};

smat_status build_plan(const HostBcsr& b, int32_t R, Plan& plan);

// Work items of one launch shape: panels whose cost exceeds max_item_frac
// of the per-worker average are split into parts (stage ranges) of about
// that size; the items are then assigned to `workers` queues. n_split =
// split panels, n_slabs = their parts (one partial-sum slab per part and
// column tile).
void build_work_items(const Plan& pl, int32_t bh, int32_t workers, double max_item_frac,
                      std::vector<WorkItem>& items, std::vector<int32_t>& cta_ptr,
                      std::vector<int32_t>& cta_items, int32_t& n_split, int32_t& n_slabs);

// Longest-processing-time assignment of items to `workers` queues.
void assign_items(const std::vector<double>& item_cost, int32_t workers,
                  std::vector<int32_t>& cta_ptr, std::vector<int32_t>& cta_items);

}  // namespace smat
