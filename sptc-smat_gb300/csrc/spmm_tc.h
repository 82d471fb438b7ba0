// spmm_tc.h — launch interface of the tensor-core SpMM kernels.
#pragma once

#include <cuda.h>
#include <cuda_runtime.h>

#include <cstdint>

namespace smat {

// Blocks per pipeline stage. A stage carries one chunk of A blocks (in the
// order the kernel consumes them), every packed B tile those blocks need,
// and one 16-bit metadata word per block.
constexpr int kChunkBlocks = 8;
// Metadata words per chunk (one 16-byte record field).
constexpr int kMetaStride = 8;

// Per-panel record of the device plan (8 x int32).
struct PanelInfo {
  int32_t chunk_off;  // first chunk of the panel
  int32_t nchunks;    // chunks in the panel
  int32_t nblk;       // blocks in the panel
  int32_t nucol;      // union columns (distinct block columns) of the panel
  uint32_t slot_mask; // bit s set: block row s of the panel has at least one block
  int32_t pad0, pad1, pad2;
};

// Per-chunk record (16 x int32 = 64 bytes): where its blocks are, the
// k-block index (column / 16) of each B tile it needs, and the metadata word
// of each of its blocks (zero past nblk).
struct ChunkRec {
  int32_t blk_off;   // first block (stream order)
  int32_t nblk;      // blocks in the chunk (1..kChunkBlocks)
  int32_t ntiles;    // distinct block columns = B tiles (1..kChunkBlocks)
  int32_t pad;
  int32_t kb[8];     // k-block of each tile, in order
  uint16_t meta[8];  // per block
};

// Per-block metadata (16 bits). Blocks of consecutive block rows ("slots")
// at the same block column form an MMA group: one tcgen05.mma with
// N = bh * length covers them all (their accumulators are adjacent in TMEM
// and their A blocks adjacent in shared memory). The group's first block
// carries the length; the others (and padding) carry length 0.
//   bits 0-4   slot of the group's first block row
//   bit  5     accumulate into the existing partial sums (else overwrite)
//   bits 6-7   MMA-issuing warp that owns the group (slot * 4 / R)
//   bits 8-12  group length (1..16) on the group's first block, else 0
//   bits 13-15 index of the group's B tile inside the stage
constexpr uint16_t kMetaAcc = 1u << 5;
constexpr int kMetaOwnerShift = 6, kMetaLenShift = 8, kMetaTileShift = 13;
constexpr int kMmaWarps = 4;

// Kernel arguments (one __grid_constant__ parameter).
struct SpmmArgs {
  const uint8_t* bpack;     // B in 4 KB tiles [k-block][128-column tile] (pack_b)
  const uint8_t* bpack2;    // low halves of B (split form)
  int64_t bp_ntiles;        // 128-column tiles per k-block in bpack
  const uint8_t* aval;      // A blocks in stream order, pre-swizzled (bh * 32 bytes each)
  const uint8_t* aval2;     // low halves of A (split form)
  const PanelInfo* panels;
  const ChunkRec* chunks;
  const int32_t* cta_ptr;   // [grid + 1]
  const int32_t* cta_items; // panels, per CTA
  const int32_t* row_map;   // [rows_padded] BCSR row -> C row, or -1
  void* C;
  int64_t ldc;
  int32_t N;
  int32_t n_tiles;
  int32_t nbr;
  int32_t c_f16;
  uint32_t idesc;
  int* err;
};

bool tc_variant_supported(int bh, int R, int nsub, bool split);
int tc_ctas_per_sm(int bh, int R, int nsub, bool split);
cudaError_t tc_launch(int bh, int R, int nsub, bool split, const SpmmArgs& args, int grid,
                      cudaStream_t stream);

}  // namespace smat
