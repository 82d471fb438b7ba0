// convert.cu — prepares the dense operand B for the tensor-core SpMM.
//
// The SpMM reads B as column-major 16-bit tiles (element (k, n) at
// B[k + n*ld], the reference's layout, src/cuda_hgemm/src/mma/mmaOBT.cu:75).
// B given in another dtype or layout is converted here into caller-provided
// scratch: FP32/FP16/BF16, row- or column-major, to FP16, BF16, or the hi+lo
// BF16 pair of the split form (hi = bf16(b), lo = bf16(b - hi)).
#include <cuda_bf16.h>
#include <cuda_fp16.h>
#include <cuda_runtime.h>

#include <cstdint>

#include "convert.h"

namespace smat {
namespace dev {

enum : int { OUT_F16 = 0, OUT_BF16 = 1, OUT_SPLIT = 2 };

template <typename T>
__device__ __forceinline__ float load_f(const T* p);
template <>
__device__ __forceinline__ float load_f<float>(const float* p) {
  return __ldg(p);
}
template <>
__device__ __forceinline__ float load_f<__half>(const __half* p) {
  return __half2float(__ldg(p));
}
template <>
__device__ __forceinline__ float load_f<__nv_bfloat16>(const __nv_bfloat16* p) {
  return __bfloat162float(__ldg(p));
}

template <int OUT>
__device__ __forceinline__ void store_out(uint16_t* hi, uint16_t* lo, int64_t off, float x) {
  if (OUT == OUT_F16) {
    hi[off] = __half_as_ushort(__float2half_rn(x));
  } else {
    const __nv_bfloat16 h = __float2bfloat16_rn(x);
    hi[off] = __bfloat16_as_ushort(h);
    if (OUT == OUT_SPLIT) lo[off] = __bfloat16_as_ushort(__float2bfloat16_rn(x - __bfloat162float(h)));
  }
}

// Column-major input: (k, n) at in[k + n*ldi]. One thread per element, k fastest.
template <typename T, int OUT>
__global__ void convert_colmajor(const T* __restrict__ in, int64_t ldi, uint16_t* __restrict__ hi,
                                 uint16_t* __restrict__ lo, int64_t ldo, int64_t K, int64_t N) {
  const int64_t total = K * N;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < total;
       i += (int64_t)gridDim.x * blockDim.x) {
    const int64_t n = i / K, k = i - n * K;
    store_out<OUT>(hi, lo, k + n * ldo, load_f<T>(in + k + n * ldi));
  }
}

// Row-major input: (k, n) at in[k*ldi + n]. 32 x 32 tiles through shared
// memory so that both the reads (along n) and the writes (along k) coalesce.
template <typename T, int OUT>
__global__ void convert_rowmajor(const T* __restrict__ in, int64_t ldi, uint16_t* __restrict__ hi,
                                 uint16_t* __restrict__ lo, int64_t ldo, int64_t K, int64_t N) {
  __shared__ float tile[32][33];
  const int64_t k0 = (int64_t)blockIdx.y * 32, n0 = (int64_t)blockIdx.x * 32;
  const int tx = threadIdx.x, ty = threadIdx.y;  // 32 x 8
  for (int r = ty; r < 32; r += 8) {
    const int64_t k = k0 + r, n = n0 + tx;
    tile[r][tx] = (k < K && n < N) ? load_f<T>(in + k * ldi + n) : 0.0f;
  }
  __syncthreads();
  for (int c = ty; c < 32; c += 8) {
    const int64_t n = n0 + c, k = k0 + tx;
    if (k < K && n < N) store_out<OUT>(hi, lo, k + n * ldo, tile[tx][c]);
  }
}

template <typename T, int OUT>
static cudaError_t run(const void* in, int layout, int64_t ldi, uint16_t* hi, uint16_t* lo,
                       int64_t ldo, int64_t K, int64_t N, cudaStream_t s) {
  if (K == 0 || N == 0) return cudaSuccess;
  if (layout == 1) {
    const int64_t total = K * N;
    int64_t blocks = (total + 255) / 256;
    if (blocks > 152 * 32) blocks = 152 * 32;
    convert_colmajor<T, OUT><<<(unsigned)blocks, 256, 0, s>>>((const T*)in, ldi, hi, lo, ldo, K, N);
  } else {
    dim3 grid((unsigned)((N + 31) / 32), (unsigned)((K + 31) / 32));
    convert_rowmajor<T, OUT><<<grid, dim3(32, 8), 0, s>>>((const T*)in, ldi, hi, lo, ldo, K, N);
  }
  return cudaGetLastError();
}

}  // namespace dev

cudaError_t convert_b(const void* in, int in_dtype, int layout, int64_t ldi, int out_mode,
                      uint16_t* hi, uint16_t* lo, int64_t ldo, int64_t K, int64_t N,
                      cudaStream_t s) {
  using namespace dev;
#define SMAT_CONV(T)                                                                  \
  switch (out_mode) {                                                                 \
    case OUT_F16: return run<T, OUT_F16>(in, layout, ldi, hi, lo, ldo, K, N, s);     \
    case OUT_BF16: return run<T, OUT_BF16>(in, layout, ldi, hi, lo, ldo, K, N, s);   \
    case OUT_SPLIT: return run<T, OUT_SPLIT>(in, layout, ldi, hi, lo, ldo, K, N, s); \
    default: return cudaErrorInvalidValue;                                            \
  }
  switch (in_dtype) {
    case 0: SMAT_CONV(float)
    case 1: SMAT_CONV(__half)
    case 2: SMAT_CONV(__nv_bfloat16)
    default: return cudaErrorInvalidValue;
  }
#undef SMAT_CONV
}

}  // namespace smat
