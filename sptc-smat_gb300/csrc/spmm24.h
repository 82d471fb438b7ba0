// spmm24.h — the structured-sparse (2:4) tensor-core path: data layout of
// its device stream and its launch interface.
//
// Blocks that are exactly 2:4 (every group of four consecutive columns of
// every row holds at most two nonzeros, judged on the FP16 values) leave the
// dense plan and go here. tcgen05.mma.sp takes the sparsity on its A operand
// (M x K), so this path computes C = A * B in the direct orientation: a
// GROUP of 8 consecutive block rows (128 rows, M = 128) times one 32-column
// WINDOW of B (K = 32, two 16-column blocks per row), N = 128 columns of C per
// pass. A UNIT is a (group, window) pair with at least one exact-2:4 block;
// its A operand is 128 rows x 16 kept values (the compressed form), in which
// the rows of block rows without a 2:4 block in the window are zero.
//
// The stream keeps only the blocks that exist: per block 16 rows x 8 kept
// FP16 values (256 bytes) and 16 rows x 16 bits of metadata (32 bytes; per
// group of four columns, the two kept columns' indices, 2 bits each, lower
// index in the lower bits, groups in column order from bit 0). The kernel's
// converter warps expand a unit into the zero-filled A tile in shared memory
// and its metadata into tensor memory.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>

namespace smat {

constexpr int kSp24GroupRows = 8;      // block rows per group (M = 128)
constexpr int kSp24StageUnits = 16;    // units per stage, at most
constexpr int kSp24StageBlocks = 32;   // blocks per stage, at most
constexpr int kSp24BlockBytes = 256 + 32;

// A unit (16 bytes): its window, blocks and where they are in the stage.
struct Sp24Unit {
  int32_t window;    // 32-column window index (columns 32 * window ..)
  uint16_t mask;     // bit 2 j + h: block row j of the group has a 2:4 block in half h of the window
  uint16_t first;    // index of its first block inside the stage (blocks in mask bit order)
  int32_t pad[2];
};

// A stage (32 bytes): consecutive units of one group, brought by one copy:
//   [nunits Sp24Unit][nblk x 256 B values][nblk x 32 B metadata]
struct Sp24Stage {
  int64_t off;       // byte offset in the stream
  int32_t bytes;     // multiple of 16
  int32_t nunits;
  int32_t nblk;
  int32_t unit0;     // index of its first unit in the group's unit list (for the B copies)
  int32_t pad[2];
};

// A group (32 bytes): its stages and units.
struct Sp24Group {
  int32_t stage0, nstages;
  int32_t unit0, nunits;    // units in the device unit-window array
  int32_t group;            // group index (block rows 8 * group ..)
  uint32_t row_mask;        // bit j: block row j has a 2:4 block
  int32_t pad[2];
};

struct Sp24Args {
  const uint8_t* stream;      // stage data
  const Sp24Stage* stages;
  const Sp24Group* groups;    // in the order the CTAs take them
  const int32_t* unit_window; // window of every unit, group by group
  const int32_t* row_map;     // [rows_padded] BCSR row -> C row (or -1)
  const uint8_t* bpack64;     // B in 8 KB tiles [128-column tile][window]: 128 rows (n) x 32 k, 64-byte swizzle
  int64_t kw;                 // windows per 128-column tile in bpack64
  void* C;
  int64_t ldc;
  int32_t N, n_tiles;
  int32_t n_groups;
  int32_t c_f16;
  uint32_t idesc;             // sparse instruction descriptor without N
  int32_t pad_;
  int* err;
  uint64_t wait_ns;
};

cudaError_t sp24_launch(const Sp24Args& args, int grid, cudaStream_t stream);
int sp24_threads();

}  // namespace smat
