// spmm_tc.cu — block-sparse x dense SpMM on sm_103a tensor cores.
//
// The reference computes each 16 x 8 tile of C with one warp and mma.sync,
// re-reading every A block ceil(N/8) times (src/cuda_hgemm/src/mma/mmaOBT.cu:18-158).
// Here one CTA owns a PANEL of R consecutive block rows and a 128*NSUB-wide
// column tile of C, and computes the transposed product
//
//     C[rows of block row r, n-tile]^T  +=  B[col : col+16, n-tile]^T * A_blk^T
//
// with tcgen05.mma (M = 128 dense columns of B, N = bh rows of the block,
// K = 16 = bw), accumulating in FP32 in tensor memory: R*NSUB accumulators of
// 128 lanes x bh columns per buffer, double buffered.
//
// Blocks of a panel are visited in order of their block column (the panel's
// "union columns"): the B tile of a column is TMA-loaded ONCE and used by
// every block row of the panel that has a block there. Every A block is read
// from HBM once per N tile.
//
// Roles (192 threads):
//   warp 0, lane 0  TMA producer: B tiles into an NB-deep ring, A blocks into
//                   an NA-deep ring, plus a small descriptor per A stage.
//   warp 1          allocates / frees TMEM; lane 0 issues the MMAs.
//   warps 2..5      epilogue: tcgen05.ld -> row scatter through row_map ->
//                   FP32 or FP16 stores of C (coalesced along N).
//
// Every wait is bounded (see tc_ptx.cuh); on a timeout the kernel raises the
// CTA's abort flag, records the site in the global error word, lets the
// producer wait for its own copies in flight and the MMA thread for its own
// MMAs, frees TMEM and returns.
#include <cuda.h>
#include <cuda_bf16.h>
#include <cuda_fp16.h>
#include <cuda_runtime.h>

#include <cstdint>

#include "spmm_tc.h"
#include "tc_ptx.cuh"

namespace smat {
namespace dev {

enum : int { KIND_PLAIN = 0, KIND_SPLIT = 1 };

// Error sites recorded in the global error word.
enum : int {
  ERR_PROD_B = 101,
  ERR_PROD_A = 102,
  ERR_PROD_END = 103,
  ERR_MMA_ACC = 201,
  ERR_MMA_A = 202,
  ERR_MMA_B = 203,
  ERR_EPI = 301,
  ERR_DRAIN = 401
};

template <int BH, int R, int NSUB, int KIND>
struct Cfg {
  static constexpr int BN = 128 * NSUB;                 // C columns per tile
  static constexpr int NOPS = (KIND == KIND_SPLIT) ? 2 : 1;
  static constexpr int NA = 32;                         // A stages
  static constexpr int NB = (NSUB * NOPS >= 2) ? 4 : 6; // B stages
  static constexpr uint32_t A_STAGE = BH * 32 * NOPS;   // bytes
  static constexpr uint32_t B_STAGE = BN * 32 * NOPS;
  static constexpr uint32_t ACC_COLS = R * NSUB * BH;   // TMEM columns per buffer
  static constexpr uint32_t TMEM_COLS = 2 * ACC_COLS;
  static constexpr uint32_t SMEM_B = NB * B_STAGE;
  static constexpr uint32_t SMEM_A = NA * A_STAGE;
  static constexpr uint32_t SMEM_BARS = 8 * (2 * NA + 2 * NB + 5);
  static constexpr uint32_t SMEM_BYTES = 1024 + SMEM_B + SMEM_A + SMEM_BARS + 4 * NA + 16;
  static_assert(TMEM_COLS >= 32 && TMEM_COLS <= 512 && (TMEM_COLS & (TMEM_COLS - 1)) == 0,
                "TMEM allocation must be a power of two in [32, 512]");
  static_assert(BH == 16 || BH == 32, "block height");
  static_assert(R <= 32, "slot field is 5 bits");
};

// Wait used only while draining after an abort: bounded, ignores the flag.
__device__ __noinline__ bool mbar_wait_drain(uint32_t bar, uint32_t parity, int* err) {
  const uint64_t t0 = globaltimer();
  while (!mbar_try_wait(bar, parity)) {
    if (globaltimer() - t0 > kWaitTimeoutNs) {
      atomicCAS(err, 0, ERR_DRAIN);
      return false;
    }
  }
  return true;
}

template <int BH, int R, int NSUB, int KIND>
__global__ void __launch_bounds__(192, 1) spmm_tc_kernel(const __grid_constant__ SpmmArgs args) {
  using C = Cfg<BH, R, NSUB, KIND>;
  extern __shared__ uint8_t smem_raw[];
  uint8_t* smem = reinterpret_cast<uint8_t*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) &
                                             ~static_cast<uintptr_t>(1023));
  uint8_t* sB = smem;
  uint8_t* sA = sB + C::SMEM_B;
  uint64_t* bars = reinterpret_cast<uint64_t*>(sA + C::SMEM_A);
  uint64_t* afull = bars;
  uint64_t* aempty = afull + C::NA;
  uint64_t* bfull = aempty + C::NA;
  uint64_t* bempty = bfull + C::NB;
  uint64_t* accfull = bempty + C::NB;
  uint64_t* accempty = accfull + 2;
  uint64_t* drainbar = accempty + 2;
  uint32_t* sdesc = reinterpret_cast<uint32_t*>(drainbar + 1);
  uint32_t* tmem_slot = sdesc + C::NA;
  volatile int* abort_flag = reinterpret_cast<volatile int*>(tmem_slot + 1);

  const int warp = threadIdx.x >> 5;
  const int lane = threadIdx.x & 31;

  if (threadIdx.x == 0) {
    for (int i = 0; i < C::NA; i++) {
      mbar_init(smem_u32(&afull[i]), 1);
      mbar_init(smem_u32(&aempty[i]), 1);
    }
    for (int i = 0; i < C::NB; i++) {
      mbar_init(smem_u32(&bfull[i]), 1);
      mbar_init(smem_u32(&bempty[i]), 1);
    }
    for (int i = 0; i < 2; i++) {
      mbar_init(smem_u32(&accfull[i]), 1);
      mbar_init(smem_u32(&accempty[i]), 4);
    }
    mbar_init(smem_u32(drainbar), 1);
    *abort_flag = 0;
    fence_barrier_init();
    prefetch_tensormap(&args.tmA);
    prefetch_tensormap(&args.tmB);
    if (KIND == KIND_SPLIT) {
      prefetch_tensormap(&args.tmA2);
      prefetch_tensormap(&args.tmB2);
    }
  }
  if (warp == 1) {
    tmem_alloc(smem_u32(tmem_slot), C::TMEM_COLS);
    tmem_relinquish();
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = *tmem_slot;

  const int it0 = args.cta_ptr[blockIdx.x];
  const int it1 = args.cta_ptr[blockIdx.x + 1];
  const int n_tiles = args.n_tiles;
  int* err = args.err;

  if (warp == 0) {
    if (lane == 0) {
      // ------------------------------------------------------------ producer
      uint32_t ai = 0, bi = 0;
      bool ok = true;
      const uint32_t sA0 = smem_u32(sA), sB0 = smem_u32(sB);
      for (int it = it0; it < it1 && ok; ++it) {
        const int panel = args.cta_items[it];
        const int u0 = args.ucol_ptr[panel], u1 = args.ucol_ptr[panel + 1];
        for (int nt = 0; nt < n_tiles && ok; ++nt) {
          const int n0 = nt * C::BN;
          uint32_t touched = 0;
          for (int u = u0; u < u1 && ok; ++u) {
            const int col = args.ucol[u];
            const uint32_t sb = bi % C::NB;
            if (!mbar_wait(smem_u32(&bempty[sb]), ((bi / C::NB) & 1) ^ 1, abort_flag, err, ERR_PROD_B)) {
              ok = false;
              break;
            }
            const uint32_t bf = smem_u32(&bfull[sb]);
            mbar_arrive_expect_tx(bf, C::B_STAGE);
            tma_load_2d(sB0 + sb * C::B_STAGE, &args.tmB, col, n0, bf);
            if (KIND == KIND_SPLIT)
              tma_load_2d(sB0 + sb * C::B_STAGE + C::BN * 32, &args.tmB2, col, n0, bf);
            ++bi;
            const int e0 = args.ublk_ptr[u], e1 = args.ublk_ptr[u + 1];
            for (int e = e0; e < e1; ++e) {
              const uint32_t v = args.ublk[e];
              const uint32_t blk = v >> 5, slot = v & 31u;
              const uint32_t sa = ai % C::NA;
              if (!mbar_wait(smem_u32(&aempty[sa]), ((ai / C::NA) & 1) ^ 1, abort_flag, err, ERR_PROD_A)) {
                ok = false;
                break;
              }
              sdesc[sa] = slot | (((touched >> slot) & 1u) << 8) | ((e == e0 ? 1u : 0u) << 9) |
                          ((e == e1 - 1 ? 1u : 0u) << 10);
              touched |= 1u << slot;
              const uint32_t af = smem_u32(&afull[sa]);
              mbar_arrive_expect_tx(af, C::A_STAGE);
              tma_load_2d(sA0 + sa * C::A_STAGE, &args.tmA, 0, (int32_t)(blk * BH), af);
              if (KIND == KIND_SPLIT)
                tma_load_2d(sA0 + sa * C::A_STAGE + BH * 32, &args.tmA2, 0, (int32_t)(blk * BH), af);
              ++ai;
            }
          }
          if (!ok) break;
          const uint32_t sa = ai % C::NA;
          if (!mbar_wait(smem_u32(&aempty[sa]), ((ai / C::NA) & 1) ^ 1, abort_flag, err, ERR_PROD_END)) {
            ok = false;
            break;
          }
          sdesc[sa] = 1u << 31;  // end of work item
          mbar_arrive(smem_u32(&afull[sa]));
          ++ai;
        }
      }
      if (!ok) {
        // wait for this thread's own copies still in flight
        for (uint32_t k = (ai > (uint32_t)C::NA ? ai - C::NA : 0); k < ai; ++k)
          mbar_wait_drain(smem_u32(&afull[k % C::NA]), (k / C::NA) & 1, err);
        for (uint32_t k = (bi > (uint32_t)C::NB ? bi - C::NB : 0); k < bi; ++k)
          mbar_wait_drain(smem_u32(&bfull[k % C::NB]), (k / C::NB) & 1, err);
      }
    }
  } else if (warp == 1) {
    if (lane == 0) {
      // ------------------------------------------------------------ MMA issuer
      const uint32_t idesc = args.idesc;
      uint32_t ai = 0, bi = 0, k = 0;
      bool ok = true, issued = false;
      const uint32_t sA0 = smem_u32(sA), sB0 = smem_u32(sB);
      for (int it = it0; it < it1 && ok; ++it) {
        for (int nt = 0; nt < n_tiles && ok; ++nt, ++k) {
          const uint32_t buf = k & 1;
          const uint32_t dbase = tmem + buf * C::ACC_COLS;
          if (!mbar_wait(smem_u32(&accempty[buf]), ((k >> 1) & 1) ^ 1, abort_flag, err, ERR_MMA_ACC)) {
            ok = false;
            break;
          }
          tc_fence_after();
          while (true) {
            const uint32_t sa = ai % C::NA;
            if (!mbar_wait(smem_u32(&afull[sa]), (ai / C::NA) & 1, abort_flag, err, ERR_MMA_A)) {
              ok = false;
              break;
            }
            const uint32_t d = sdesc[sa];
            if (d >> 31) {
              mbar_arrive(smem_u32(&aempty[sa]));
              ++ai;
              umma_commit(smem_u32(&accfull[buf]));
              break;
            }
            const uint32_t sb = bi % C::NB;
            if (d & (1u << 9)) {
              if (!mbar_wait(smem_u32(&bfull[sb]), (bi / C::NB) & 1, abort_flag, err, ERR_MMA_B)) {
                ok = false;
                break;
              }
            }
            tc_fence_after();
            const uint32_t slot = d & 31u, acc = (d >> 8) & 1u;
            const uint32_t a_addr = sA0 + sa * C::A_STAGE;
            const uint32_t b_addr = sB0 + sb * C::B_STAGE;
            const uint64_t a_hi = desc_kmajor_sw32(a_addr);
#pragma unroll
            for (int j = 0; j < NSUB; ++j) {
              const uint32_t dcol = dbase + slot * (NSUB * BH) + j * BH;
              const uint64_t b_hi = desc_kmajor_sw32(b_addr + j * 128 * 32);
              umma_f16(dcol, b_hi, a_hi, idesc, acc);
              if (KIND == KIND_SPLIT) {
                const uint64_t a_lo = desc_kmajor_sw32(a_addr + BH * 32);
                const uint64_t b_lo = desc_kmajor_sw32(b_addr + C::BN * 32 + j * 128 * 32);
                umma_f16(dcol, b_hi, a_lo, idesc, 1);
                umma_f16(dcol, b_lo, a_hi, idesc, 1);
              }
            }
            issued = true;
            umma_commit(smem_u32(&aempty[sa]));
            if (d & (1u << 10)) {
              umma_commit(smem_u32(&bempty[sb]));
              ++bi;
            }
            ++ai;
          }
        }
      }
      if (!ok && issued) {
        umma_commit(smem_u32(drainbar));
        mbar_wait_drain(smem_u32(drainbar), 0, err);
      }
    }
  } else {
    // -------------------------------------------------------------- epilogue
    const uint32_t q = warp & 3;  // TMEM lane quadrant this warp may access
    uint32_t k = 0;
    bool ok = true;
    for (int it = it0; it < it1 && ok; ++it) {
      const int panel = args.cta_items[it];
      for (int nt = 0; nt < n_tiles; ++nt, ++k) {
        const uint32_t buf = k & 1;
        if (!mbar_wait(smem_u32(&accfull[buf]), (k >> 1) & 1, abort_flag, err, ERR_EPI)) {
          ok = false;
          break;
        }
        tc_fence_after();
        const uint32_t dbase = tmem + ((q * 32u) << 16) + buf * C::ACC_COLS;
        for (int s = 0; s < R; ++s) {
          const int rb = panel * R + s;
          if (rb >= args.nbr) break;
          const bool empty = args.rowptr[rb + 1] == args.rowptr[rb];
          const int myrow = lane < BH ? args.row_map[(int64_t)rb * BH + lane] : -1;
#pragma unroll
          for (int j = 0; j < NSUB; ++j) {
            const int n = nt * C::BN + j * 128 + (int)q * 32 + lane;
#pragma unroll
            for (int h = 0; h < BH; h += 16) {
              float v[16];
              if (!empty) {
                tmem_ld_x16(dbase + s * (NSUB * BH) + j * BH + h, v);
              } else {
#pragma unroll
                for (int m = 0; m < 16; ++m) v[m] = 0.0f;
              }
#pragma unroll
              for (int m = 0; m < 16; ++m) {
                const int row = __shfl_sync(0xffffffffu, myrow, h + m);
                if (row >= 0 && n < args.N) {
                  const int64_t off = (int64_t)row * args.ldc + n;
                  if (args.c_f16)
                    __stcs(reinterpret_cast<__half*>(args.C) + off, __float2half_rn(v[m]));
                  else
                    __stcs(reinterpret_cast<float*>(args.C) + off, v[m]);
                }
              }
            }
          }
        }
        tc_fence_before();
        __syncwarp();
        if (lane == 0) mbar_arrive(smem_u32(&accempty[buf]));
      }
    }
  }

  tc_fence_before();
  __syncthreads();
  if (warp == 1) {
    tc_fence_after();
    tmem_dealloc(tmem, C::TMEM_COLS);
  }
}

template <int BH, int R, int NSUB, int KIND>
static cudaError_t launch_one(const SpmmArgs& args, int grid, cudaStream_t stream) {
  using C = Cfg<BH, R, NSUB, KIND>;
  auto kfn = spmm_tc_kernel<BH, R, NSUB, KIND>;
  cudaError_t e = cudaFuncSetAttribute(kfn, cudaFuncAttributeMaxDynamicSharedMemorySize, C::SMEM_BYTES);
  if (e != cudaSuccess) return e;
  kfn<<<grid, 192, C::SMEM_BYTES, stream>>>(args);
  return cudaGetLastError();
}

template <int BH, int R, int NSUB, int KIND>
static int ctas_per_sm_one() {
  using C = Cfg<BH, R, NSUB, KIND>;
  int by_tmem = 512 / C::TMEM_COLS;
  int by_smem = (227 * 1024) / (C::SMEM_BYTES + 1024);
  int n = by_tmem < by_smem ? by_tmem : by_smem;
  return n < 1 ? 1 : (n > 4 ? 4 : n);
}

}  // namespace dev

#define SMAT_TC_VARIANTS(X) \
  X(16, 4, 1, 0)            \
  X(16, 8, 1, 0)            \
  X(16, 16, 1, 0)           \
  X(16, 4, 2, 0)            \
  X(16, 8, 2, 0)            \
  X(32, 4, 1, 0)            \
  X(32, 8, 1, 0)            \
  X(32, 4, 2, 0)            \
  X(16, 4, 1, 1)            \
  X(16, 8, 1, 1)            \
  X(16, 16, 1, 1)           \
  X(16, 4, 2, 1)            \
  X(16, 8, 2, 1)            \
  X(32, 4, 1, 1)            \
  X(32, 8, 1, 1)            \
  X(32, 4, 2, 1)

bool tc_variant_supported(int bh, int R, int nsub, bool split) {
#define SMAT_TC_MATCH(BH, R_, NS, K) \
  if (bh == BH && R == R_ && nsub == NS && (split ? 1 : 0) == K) return true;
  SMAT_TC_VARIANTS(SMAT_TC_MATCH)
#undef SMAT_TC_MATCH
  return false;
}

int tc_ctas_per_sm(int bh, int R, int nsub, bool split) {
#define SMAT_TC_OCC(BH, R_, NS, K) \
  if (bh == BH && R == R_ && nsub == NS && (split ? 1 : 0) == K) return dev::ctas_per_sm_one<BH, R_, NS, K>();
  SMAT_TC_VARIANTS(SMAT_TC_OCC)
#undef SMAT_TC_OCC
  return 1;
}

cudaError_t tc_launch(int bh, int R, int nsub, bool split, const SpmmArgs& args, int grid,
                      cudaStream_t stream) {
#define SMAT_TC_LAUNCH(BH, R_, NS, K)                             \
  if (bh == BH && R == R_ && nsub == NS && (split ? 1 : 0) == K) \
    return dev::launch_one<BH, R_, NS, K>(args, grid, stream);
  SMAT_TC_VARIANTS(SMAT_TC_LAUNCH)
#undef SMAT_TC_LAUNCH
  return cudaErrorInvalidValue;
}

}  // namespace smat
