// spmm_tc.h — launch interface of the tensor-core SpMM kernels.
#pragma once

#include <cuda.h>
#include <cuda_runtime.h>

#include <cstdint>

namespace smat {

// Kernel arguments (passed as one __grid_constant__ parameter so that the
// tensor maps stay in parameter space).
struct SpmmArgs {
  CUtensorMap tmA;   // A blocks: 2-D [nnzb * bh rows][16 cols], 16-bit, 32-byte swizzle
  CUtensorMap tmB;   // B: 2-D {K (contiguous), N}, 16-bit, 32-byte swizzle
  CUtensorMap tmA2;  // low halves of A (split form)
  CUtensorMap tmB2;  // low halves of B (split form)
  const int32_t* rowptr;    // [nbr + 1] block row pointer
  const int32_t* ucol_ptr;  // [n_panels + 1]
  const int32_t* ucol;      // union column starts
  const int32_t* ublk_ptr;  // [n_ucols + 1]
  const uint32_t* ublk;     // (block << 5) | slot
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
