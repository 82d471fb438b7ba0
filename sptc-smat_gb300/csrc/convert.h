// convert.h — B operand preparation kernels (convert.cu).
#pragma once

#include <cuda_runtime.h>

#include <cstdint>

namespace smat {

// in_dtype: 0 F32, 1 F16, 2 BF16; layout: 0 row-major (k*ldi + n), 1 column-major
// (k + n*ldi); out_mode: 0 FP16, 1 BF16, 2 hi+lo BF16 (lo may not be NULL).
// Output is column-major with leading dimension ldo.
cudaError_t convert_b(const void* in, int in_dtype, int layout, int64_t ldi, int out_mode,
                      uint16_t* hi, uint16_t* lo, int64_t ldo, int64_t K, int64_t N,
                      cudaStream_t s);

}  // namespace smat
