// spmm_tc.h — launch interface of the tensor-core SpMM kernels and the
// layout of their device work plan.
#pragma once

#include <cuda.h>
#include <cuda_runtime.h>

#include <cstdint>

namespace smat {

// A pipeline STAGE carries up to stage_rows(cls) / bh A blocks of one panel
// (in the order the kernel consumes them), up to stage_tiles(cls) packed B
// tiles those blocks need, and the stage's MMA list. There are four stage
// shapes ("plan classes"), each the largest that still leaves three stages
// in flight in shared memory: class 0 for the FP16 and BF16 forms (28
// blocks of 16 rows and 14 B tiles: 14 KB of A and 56 KB of B), class 1
// for the split form, whose stages hold hi and lo copies of everything (14
// blocks and 7 tiles: the same bytes), class 2 for the FP8 form, whose
// stages also stage the e4m3 blocks before conversion (24 blocks, 12
// tiles), class 3 for the FP16 and BF16 forms with 256-column B tiles (N >
// 128 in one pass over A: 14 blocks and 7 tiles of 8 KB).
constexpr int kPlanClasses = 4;
constexpr int kMaxStageTiles = 16;   // StageRec::kb capacity (a copy warp issues at most two copies)
constexpr int kMaxStageBlocks = 31;  // the entry's position field has 5 bits
__host__ __device__ constexpr int stage_rows(int cls) { return cls == 0 ? 448 : (cls == 2 ? 384 : 224); }
__host__ __device__ constexpr int stage_tiles(int cls) { return cls == 0 ? 14 : (cls == 2 ? 12 : 7); }
constexpr int kMmaWarps = 4;      // MMA-issuing warps; each owns a quarter of a panel's TMEM slots
constexpr int kMinCutBlocks = 16; // a block row is cut over the issuing warps only from this many blocks
constexpr int kMaxGroupN = 256;   // widest tcgen05.mma N (kind::f16, M = 128)

// Per-panel record (8 x int32).
struct PanelInfo {
  int32_t stage_off;   // first stage of the panel
  int32_t nstages;     // stages of the panel
  int32_t nblk;        // blocks in the panel
  int32_t nucol;       // distinct block columns of the panel
  uint32_t slot_mask;  // bit s set: slot s of the panel has at least one block
  uint32_t ext_mask;   // bit s set: slot s holds a later part of the row in slot s - R / kMmaWarps
  int32_t pad1, pad2;
};

// Per-stage record (96 bytes), read by the copy warps. In the device A
// stream of a form (ABLK = bh * 32 bytes per block and operand, NOPS = 2 for
// the split form, else 1) a stage occupies
//     [nblk * ABLK blocks (hi)][nblk * ABLK blocks (lo, split form only)][header]
// starting at byte blk_off * ABLK * NOPS + hdr_off, where hdr_off is the sum
// of the header bytes of all earlier stages. In the FP8 stream (16 x 16
// blocks) a stage occupies
//     [nblk * 256 e4m3 blocks][nblk FP32 scales, padded to 16 bytes][header]
// starting at byte blk_off * 256 + scl_off + hdr_off, where scl_off is the
// sum of the padded scale bytes of all earlier stages.
struct StageRec {
  int64_t blk_off;     // blocks before this stage (stream order)
  int64_t hdr_off;     // header bytes before this stage
  int32_t nblk;        // A blocks in the stage
  int32_t hdr_bytes;   // bytes of this stage's header (multiple of 16)
  int32_t ntiles;      // B tiles (distinct block columns) of the stage, 1..stage_tiles
  int32_t scl_off;     // padded FP8 scale bytes before this stage
  int32_t kb[kMaxStageTiles];  // k-block (column / 16) of each tile
};

// Padded bytes of the FP32 scales of n FP8 blocks.
__host__ __device__ constexpr int fp8_scale_bytes(int n) { return (4 * n + 15) / 16 * 16; }

// Stage header (little-endian), kStageHdrFixed bytes then one 32-bit entry
// per MMA group, grouped by issuing warp:
//   uint16 warp_list[4]   bits 0-7 first entry of warp w, bits 8-15 its entry count
//   uint16 nblk, ntiles, pad[2]
//   uint32 entry[...]
// A group is a run of consecutive block rows ("slots") with a block at the
// same block column, the same accumulate flag and the same owner; it is one
// tcgen05.mma with N = bh * len (its accumulators are adjacent in TMEM and
// its A blocks adjacent in the stage). Entry bits:
//   0-4 position of the first A block in the stage, 5-8 B tile in the stage,
//   9-13 first slot, 14-17 len - 1, 18 accumulate (else overwrite).
constexpr int kStageHdrFixed = 16;
constexpr uint32_t kEntAccBit = 1u << 18;
// Largest header of a stage with sb blocks (one entry per block at most).
__host__ __device__ constexpr int stage_hdr_max(int sb) { return kStageHdrFixed + 4 * sb; }

// A unit of work of one CTA: stages [s0, s1) of a panel. A panel whose
// stages are split over several items ("parts", for load balance) has a
// split index: its parts write partial sums to workspace slabs, and the part
// that finishes last (an atomic counter per split panel and column tile)
// adds the slabs and writes C.
struct WorkItem {
  int32_t panel;
  int32_t s0, s1;      // stage range, relative to the panel's first stage
  int32_t split;       // -1: the whole panel; else index of the split panel
  int32_t part;        // part number within the split panel
  int32_t nparts;      // parts of the split panel
  int32_t slab;        // first slab of the split panel (one per part and column tile)
  int32_t prob;        // problem of a grouped launch (0 for a single SpMM)
};

// Everything the kernel needs about one SpMM problem.
struct ProblemDesc {
  const uint8_t* bpack;      // B in 4 KB tiles [128-column tile][k-block] (pack_b); the split
                             // form stores [hi tile | lo tile] pairs, 8 KB per tile
  int64_t bp_kbs;            // k-blocks per 128-column tile in bpack ([column tile][k-block])
  const uint8_t* aval;       // A stream of the form (see StageRec)
  const PanelInfo* panels;
  const StageRec* stages;
  const int32_t* row_map;    // [panels * R * bh] plan row -> C row, or -1
  void* C;
  int64_t ldc;
  float* slabs;              // partial sums of split panels: [slab][R * bh rows][BN] FP32
  int32_t* counters;         // [split panels][column tiles][4], zero before the launch
  int32_t N;
  int32_t n_tiles;
  int32_t nbr;               // plan block rows: panels * R (TMEM slots)
  int32_t c_f16;
  uint32_t idesc;            // instruction descriptor without the N field
  int32_t pad[3];
};

// Kernel arguments (one __grid_constant__ parameter). A single SpMM passes
// its problem by value (one); a grouped launch passes a device array
// (probs, indexed by WorkItem::prob).
// A launch: its problems and work items. CTA b takes the items order[b],
// then order[grid + atomicAdd(next_item, 1)], ... until the list is done:
// the items are sorted by decreasing estimated cost, so whichever CTA is
// free first takes the largest item left (the counter is zero at launch).
// wait_ns bounds every device-side wait (0: 4 s); stall_stage k > 0 makes
// the first MMA-issuing thread of CTA 0 wait, before its k-th stage, on a
// barrier nothing arrives at (a test of the bounded-wait error path);
// depth >= 2 caps the stage slots in flight (the pipeline depth; 0: all
// that fit in shared memory).
struct SpmmArgs {
  ProblemDesc one;
  const ProblemDesc* probs;
  const int32_t* order;      // [n_items] item indices by decreasing cost
  int32_t* next_item;        // zero at launch
  const WorkItem* items;
  int* err;
  int32_t n_items;
  int32_t stall_stage;
  uint64_t wait_ns;
  int32_t depth;
  int32_t pad_;
};

// Kernel kinds: 0 plain (FP16 or BF16 A and B), 1 split hi+lo BF16, 2 FP8 A
// (e4m3 + per-block scale, converted to FP16 in shared memory).
enum : int { TC_KIND_PLAIN = 0, TC_KIND_SPLIT = 1, TC_KIND_FP8 = 2 };
bool tc_variant_supported(int bh, int R, int nsub, int kind);
int tc_ctas_per_sm(int bh, int R, int nsub, int kind);
cudaError_t tc_launch(int bh, int R, int nsub, int kind, const SpmmArgs& args, int grid,
                      cudaStream_t stream);

}  // namespace smat
