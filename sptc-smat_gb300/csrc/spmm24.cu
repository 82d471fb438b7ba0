// spmm24.cu — C += A24 * B for the exact-2:4 blocks, on the structured-sparse
// tensor cores (tcgen05.mma.sp, kind::f16: M = 128 rows, N = 128 columns,
// K = 32 with A stored as 128 x 16 kept values plus 2-bit indices).
//
// The reference multiplies its 2:4 blocks with the warp-level mma.sp
// m16n8k32, one 16-row block row per warp (src/cuda_hgemm/src/mma/mmaOBTS_large.cu:19-254).
// tcgen05.mma.sp needs M = 64 or 128 rows of A, so a unit here is a group of
// 8 block rows (128 rows) times one 32-column window of B (the layout is in
// spmm24.h). It runs after the dense kernel, which writes every row of C from
// the other blocks, and adds its products into C.
//
// Roles (384 threads), one CTA per SM, groups taken round-robin from a list
// sorted by decreasing work:
//   warp 0        MMA issuer (lane 0); owns TMEM (two 128-column
//                 accumulators, then the metadata column of each A-tile
//                 slot, 64 columns apart: the MMA's metadata address is
//                 kept on a 64-column boundary).
//   warp 1        stage copies: the compact unit data (values, metadata).
//   warp 2        B copies: one 8 KB tile (32 rows of B x 128 columns,
//                 64-byte swizzle) per unit.
//   warps 4..7    epilogue: tcgen05.ld of the accumulator (lane = row) and
//                 C[row, :] += it, rows through the row map.
//   warps 8..11   converters: each thread owns one of the 128 rows of a unit,
//                 writes its 16 kept values into the zero-filled A tile in
//                 shared memory (32-byte swizzle) and its 32-bit metadata word
//                 into the unit's TMEM column (tcgen05.st).
// Waits are bounded like the dense kernel's; an expired wait aborts the CTA
// after its copies and MMAs in flight have landed.
#include <cuda.h>
#include <cuda_fp16.h>
#include <cuda_runtime.h>

#include <atomic>
#include <cstdint>

#include "spmm24.h"
#include "tc_ptx.cuh"

namespace smat {
namespace dev {

enum : int {
  ERR24_STAGE = 501,
  ERR24_B = 502,
  ERR24_CONV = 503,
  ERR24_MMA = 504,
  ERR24_EPI = 505,
  ERR24_DRAIN = 506
};

struct Sp24Cfg {
  static constexpr int NS = 4;                                   // stage slots
  static constexpr uint32_t STAGE_MAX =
      kSp24StageUnits * sizeof(Sp24Unit) + kSp24StageBlocks * kSp24BlockBytes;
  static constexpr uint32_t STAGE_SLOT = (STAGE_MAX + 1023) / 1024 * 1024;
  static constexpr int NT = 4;                                   // A tile slots (and metadata columns)
  static constexpr uint32_t ATILE = 128 * 32;                    // 128 rows x 16 kept values
  static constexpr int NBT = 12;                                 // B tile slots (8 KB copies from L2 in flight)
  static constexpr uint32_t BTILE = 128 * 64;                    // 128 columns x 32 k
  static constexpr uint32_t OFF_A = NS * STAGE_SLOT;
  static constexpr uint32_t OFF_B = OFF_A + NT * ATILE;
  static constexpr uint32_t RING = OFF_B + NBT * BTILE;
  static constexpr uint32_t NBARS = 2 * NS + 2 * NT + 2 * NBT + 4 + 1;
  static constexpr uint32_t SMEM_BYTES = 1024 + RING + 8 * NBARS + 16;
  static constexpr uint32_t META_COL0 = 256;                     // metadata column of A slot t: META_COL0 + 64 t
  static constexpr uint32_t META_STRIDE = 64;
  static constexpr uint32_t TMEM_COLS = 512;                     // 2 x 128 accumulator + NT metadata
  static constexpr int THREADS = 384;
  static_assert(STAGE_MAX % 16 == 0, "stage bytes");
  static_assert(SMEM_BYTES <= 227 * 1024, "shared memory");
  static_assert(META_COL0 + META_STRIDE * (NT - 1) < TMEM_COLS, "metadata columns inside the allocation");
};

__device__ __forceinline__ bool w24(uint32_t bar, uint32_t parity, volatile int* abort, int* err, int where,
                                    uint64_t lim) {
  return mbar_try_wait(bar, parity) || mbar_wait(bar, parity, abort, err, where, lim);
}

__device__ __forceinline__ bool w24_warp(uint32_t bar, uint32_t parity, int lane, volatile int* abort, int* err,
                                         int where, uint64_t lim) {
  int got = 1;
  if (lane == 0) got = w24(bar, parity, abort, err, where, lim) ? 1 : 0;
  return __shfl_sync(0xffffffffu, got, 0) != 0;
}

__device__ __noinline__ void drain24(uint32_t bar, uint32_t parity, int* err, uint64_t lim) {
  const uint64_t t0 = globaltimer();
  while (!mbar_try_wait(bar, parity))
    if (globaltimer() - t0 > lim) {
      atomicCAS(err, 0, ERR24_DRAIN);
      return;
    }
}

// 64-byte-swizzle K-major descriptor (rows of 64 bytes, 8-row groups 512 bytes apart).
__device__ __forceinline__ uint64_t desc_kmajor_sw64(uint32_t saddr) {
  uint64_t d = 0;
  d |= static_cast<uint64_t>((saddr & 0x3FFFFu) >> 4);
  d |= static_cast<uint64_t>(1) << 16;
  d |= static_cast<uint64_t>(512 >> 4) << 32;
  d |= static_cast<uint64_t>(1) << 46;
  d |= static_cast<uint64_t>(4) << 61;  // 64-byte swizzle
  return d;
}

__device__ __forceinline__ void umma_sp_f16(uint32_t tmem_d, uint64_t adesc, uint64_t bdesc, uint32_t tmem_meta,
                                            uint32_t idesc, uint32_t accumulate) {
  asm volatile(
      "{\n .reg .pred p;\n setp.ne.b32 p, %5, 0;\n"
      " tcgen05.mma.sp.cta_group::1.kind::f16 [%0], %1, %2, [%3], %4, p;\n}" ::"r"(tmem_d),
      "l"(adesc), "l"(bdesc), "r"(tmem_meta), "r"(idesc), "r"(accumulate)
      : "memory");
}

__device__ __forceinline__ void tmem_st_x1(uint32_t taddr, uint32_t v) {
  asm volatile("tcgen05.st.sync.aligned.32x32b.x1.b32 [%0], {%1};" ::"r"(taddr), "r"(v) : "memory");
}

__global__ void __launch_bounds__(Sp24Cfg::THREADS, 1) spmm24_kernel(const __grid_constant__ Sp24Args args) {
  using C = Sp24Cfg;
  extern __shared__ uint8_t smem_raw[];
  uint8_t* smem = reinterpret_cast<uint8_t*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) &
                                             ~static_cast<uintptr_t>(1023));
  uint64_t* s_full = reinterpret_cast<uint64_t*>(smem + C::RING);
  uint64_t* s_free = s_full + C::NS;
  uint64_t* a_ready = s_free + C::NS;
  uint64_t* a_free = a_ready + C::NT;
  uint64_t* b_full = a_free + C::NT;
  uint64_t* b_free = b_full + C::NBT;
  uint64_t* accfull = b_free + C::NBT;
  uint64_t* accempty = accfull + 2;
  uint64_t* drainbar = accempty + 2;
  uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(drainbar + 1);
  volatile int* abort_flag = reinterpret_cast<volatile int*>(tmem_slot + 1);

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const uint64_t lim = args.wait_ns ? args.wait_ns : kWaitTimeoutNs;
  int* err = args.err;

  if (threadIdx.x == 0) {
    for (int i = 0; i < C::NS; i++) {
      mbar_init(smem_u32(&s_full[i]), 1);
      mbar_init(smem_u32(&s_free[i]), 4);
    }
    for (int i = 0; i < C::NT; i++) {
      mbar_init(smem_u32(&a_ready[i]), 4);
      mbar_init(smem_u32(&a_free[i]), 1);
    }
    for (int i = 0; i < C::NBT; i++) {
      mbar_init(smem_u32(&b_full[i]), 1);
      mbar_init(smem_u32(&b_free[i]), 1);
    }
    for (int i = 0; i < 2; i++) {
      mbar_init(smem_u32(&accfull[i]), 1);
      mbar_init(smem_u32(&accempty[i]), 4);
    }
    mbar_init(smem_u32(drainbar), 1);
    *abort_flag = 0;
    fence_barrier_init();
  }
  if (warp == 0) {
    tmem_alloc(smem_u32(tmem_slot), C::TMEM_COLS);
    tmem_relinquish();
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = *tmem_slot;
  const uint32_t smem0 = smem_u32(smem);
  const int G = (int)gridDim.x;

  if (warp == 1) {
    // ---------------------------------------------------------- stage copies
    if (lane == 0) {
      uint32_t sc = 0;
      bool ok = true;
      for (int gi = blockIdx.x; gi < args.n_groups && ok; gi += G) {
        const Sp24Group g = args.groups[gi];
        for (int nt = 0; nt < args.n_tiles && ok; ++nt)
          for (int st = 0; st < g.nstages; ++st, ++sc) {
            const uint32_t slot = sc % C::NS;
            if (sc >= (uint32_t)C::NS &&
                !w24(smem_u32(&s_free[slot]), ((sc - C::NS) / C::NS) & 1, abort_flag, err, ERR24_STAGE, lim)) {
              ok = false;
              break;
            }
            const Sp24Stage s = args.stages[g.stage0 + st];
            const uint32_t fb = smem_u32(&s_full[slot]);
            mbar_arrive_expect_tx(fb, (uint32_t)s.bytes);
            bulk_load(smem0 + slot * C::STAGE_SLOT, args.stream + s.off, (uint32_t)s.bytes, fb);
          }
      }
      if (!ok) {
        const uint32_t lo = sc > (uint32_t)C::NS ? sc - C::NS : 0;
        for (uint32_t k = lo; k < sc; ++k) drain24(smem_u32(&s_full[k % C::NS]), (k / C::NS) & 1, err, lim);
      }
    }
  } else if (warp == 2) {
    // -------------------------------------------------------------- B copies
    if (lane == 0) {
      uint32_t u = 0;
      bool ok = true;
      for (int gi = blockIdx.x; gi < args.n_groups && ok; gi += G) {
        const Sp24Group g = args.groups[gi];
        for (int nt = 0; nt < args.n_tiles && ok; ++nt)
          for (int i = 0; i < g.nunits; ++i, ++u) {
            const uint32_t x = u % C::NBT;
            if (u >= (uint32_t)C::NBT &&
                !w24(smem_u32(&b_free[x]), ((u - C::NBT) / C::NBT) & 1, abort_flag, err, ERR24_B, lim)) {
              ok = false;
              break;
            }
            const int w = args.unit_window[g.unit0 + i];
            const uint32_t fb = smem_u32(&b_full[x]);
            mbar_arrive_expect_tx(fb, C::BTILE);
            bulk_load(smem0 + C::OFF_B + x * C::BTILE, args.bpack64 + ((int64_t)nt * args.kw + w) * C::BTILE,
                      C::BTILE, fb);
          }
      }
      if (!ok) {
        const uint32_t lo = u > (uint32_t)C::NBT ? u - C::NBT : 0;
        for (uint32_t k = lo; k < u; ++k) drain24(smem_u32(&b_full[k % C::NBT]), (k / C::NBT) & 1, err, lim);
      }
    }
  } else if (warp == 0) {
    // ----------------------------------------------------------------- MMAs
    if (lane == 0) {
      uint32_t u = 0, k = 0;
      bool ok = true, issued = false;
      for (int gi = blockIdx.x; gi < args.n_groups && ok; gi += G) {
        const Sp24Group g = args.groups[gi];
        for (int nt = 0; nt < args.n_tiles && ok; ++nt, ++k) {
          const uint32_t buf = k & 1;
          if (!w24(smem_u32(&accempty[buf]), (k >> 1) & 1, abort_flag, err, ERR24_MMA, lim)) {
            ok = false;
            break;
          }
          tc_fence_after();
          for (int i = 0; i < g.nunits; ++i, ++u) {
            const uint32_t t = u % C::NT, x = u % C::NBT;
            if (!w24(smem_u32(&a_ready[t]), (u / C::NT) & 1, abort_flag, err, ERR24_MMA, lim) ||
                !w24(smem_u32(&b_full[x]), (u / C::NBT) & 1, abort_flag, err, ERR24_MMA, lim)) {
              ok = false;
              break;
            }
            tc_fence_after();
            const uint64_t ad = desc_kmajor_sw32(smem0 + C::OFF_A + t * C::ATILE);
            const uint64_t bd = desc_kmajor_sw64(smem0 + C::OFF_B + x * C::BTILE);
            umma_sp_f16(tmem + buf * 128, ad, bd, tmem + C::META_COL0 + C::META_STRIDE * t, args.idesc | ((128u >> 3) << 17), i > 0 ? 1u : 0u);
            issued = true;
            umma_commit(smem_u32(&a_free[t]));
            umma_commit(smem_u32(&b_free[x]));
          }
          if (!ok) break;
          umma_commit(smem_u32(&accfull[buf]));
        }
      }
      if (!ok && issued) {
        umma_commit(smem_u32(drainbar));
        drain24(smem_u32(drainbar), 0, err, lim);
      }
    }
  } else if (warp >= 8) {
    // ------------------------------------------------------------ converters
    // Thread r (0..127) owns row r of every unit: block row j = r / 16 of the
    // group, row r % 16 of its blocks. It writes the row's 32 bytes of the A
    // tile (16 kept values: the window's first half, then its second; zeros
    // where the block row has no 2:4 block) in the 32-byte swizzle, and TMEM
    // lane r of the unit's metadata column. The sparse MMA reads metadata per
    // 16-row slab (here: one block row j): lane 16 j + 8 h + i holds the
    // 16-bit metadata of K-half h (the window's block h) for row i of the
    // slab in bits 0..15 and for row i + 8 in bits 16..31 (0x4444 for an
    // absent block: indices 0 and 1 of zero values).
    const int q = warp - 8;
    const int r = q * 32 + lane;
    const int j = r >> 4, rr = r & 15;
    uint32_t u = 0, sc = 0;
    bool ok = true;
    for (int gi = blockIdx.x; gi < args.n_groups && ok; gi += G) {
      const Sp24Group g = args.groups[gi];
      for (int nt = 0; nt < args.n_tiles && ok; ++nt)
        for (int st = 0; st < g.nstages && ok; ++st, ++sc) {
          const uint32_t slot = sc % C::NS;
          if (!w24_warp(smem_u32(&s_full[slot]), (sc / C::NS) & 1, lane, abort_flag, err, ERR24_CONV, lim)) {
            ok = false;
            break;
          }
          const int nunits = args.stages[g.stage0 + st].nunits;
          const int nblk = args.stages[g.stage0 + st].nblk;
          const uint8_t* sp = smem + slot * C::STAGE_SLOT;
          const Sp24Unit* units = reinterpret_cast<const Sp24Unit*>(sp);
          const uint8_t* vals = sp + nunits * sizeof(Sp24Unit);
          const uint8_t* metas = vals + (size_t)nblk * 256;
          for (int i = 0; i < nunits; ++i, ++u) {
            const uint32_t t = u % C::NT;
            if (u >= (uint32_t)C::NT &&
                !w24_warp(smem_u32(&a_free[t]), ((u - C::NT) / C::NT) & 1, lane, abort_flag, err, ERR24_CONV, lim)) {
              ok = false;
              break;
            }
            const uint32_t mask = units[i].mask;
            const uint32_t first = units[i].first;
            uint8_t* arow = smem + C::OFF_A + t * C::ATILE + r * 32;
#pragma unroll
            for (int h = 0; h < 2; ++h) {
              const uint32_t bit = 2u * j + h;
              uint4 v = make_uint4(0, 0, 0, 0);
              if ((mask >> bit) & 1u) {
                const uint32_t blk = first + __popc(mask & ((1u << bit) - 1u));
                v = *reinterpret_cast<const uint4*>(vals + (size_t)blk * 256 + rr * 16);
              }
              *reinterpret_cast<uint4*>(arow + ((h ^ ((r >> 2) & 1)) << 4)) = v;
            }
            uint32_t word = 0x44444444u;
            {
              const uint32_t mh = (r >> 3) & 1u, mi = r & 7u;  // K-half and slab row of this lane
              const uint32_t bit = 2u * j + mh;
              if ((mask >> bit) & 1u) {
                const uint32_t blk = first + __popc(mask & ((1u << bit) - 1u));
                const uint16_t* mp = reinterpret_cast<const uint16_t*>(metas + (size_t)blk * 32);
                word = (uint32_t)mp[mi] | ((uint32_t)mp[mi + 8] << 16);
              }
            }
            tmem_st_x1(tmem + ((uint32_t)(q * 32) << 16) + C::META_COL0 + C::META_STRIDE * t, word);
            tmem_st_wait();
            fence_proxy_async_smem();
            tc_fence_before();
            __syncwarp();
            if (lane == 0) mbar_arrive(smem_u32(&a_ready[t]));
          }
          __syncwarp();
          if (lane == 0 && ok) mbar_arrive(smem_u32(&s_free[slot]));
        }
    }
  } else if (warp >= 4) {
    // -------------------------------------------------------------- epilogue
    const int q = warp - 4;
    const int r = q * 32 + lane;
    if (lane == 0) {
      mbar_arrive(smem_u32(&accempty[0]));
      mbar_arrive(smem_u32(&accempty[1]));
    }
    uint32_t k = 0;
    bool ok = true;
    for (int gi = blockIdx.x; gi < args.n_groups && ok; gi += G) {
      const Sp24Group g = args.groups[gi];
      const int64_t prow = (int64_t)g.group * 128 + r;
      const int crow = ((g.row_mask >> (r >> 4)) & 1u) ? args.row_map[prow] : -1;
      for (int nt = 0; nt < args.n_tiles; ++nt, ++k) {
        const uint32_t buf = k & 1;
        if (!w24_warp(smem_u32(&accfull[buf]), (k >> 1) & 1, lane, abort_flag, err, ERR24_EPI, lim)) {
          ok = false;
          break;
        }
        tc_fence_after();
#pragma unroll 1
        for (int c = 0; c < 128; c += 32) {
          float v[32];
          tmem_ld_x32(tmem + ((uint32_t)(q * 32) << 16) + buf * 128 + c, v);
          if (crow >= 0) {
            const int n0 = nt * 128 + c;
            if (args.c_f16) {
              __half* cp = reinterpret_cast<__half*>(args.C) + (int64_t)crow * args.ldc + n0;
#pragma unroll
              for (int m = 0; m < 32; ++m)
                if (n0 + m < args.N) cp[m] = __float2half_rn(__half2float(cp[m]) + v[m]);
            } else {
              float* cp = reinterpret_cast<float*>(args.C) + (int64_t)crow * args.ldc + n0;
#pragma unroll
              for (int m = 0; m < 32; ++m)
                if (n0 + m < args.N) cp[m] += v[m];
            }
          }
        }
        tc_fence_before();
        __syncwarp();
        if (lane == 0) mbar_arrive(smem_u32(&accempty[buf]));
      }
    }
  }
  __syncwarp();
  tc_fence_before();
  __syncthreads();
  if (warp == 0) {
    tc_fence_after();
    tmem_dealloc(tmem, C::TMEM_COLS);
  }
}

}  // namespace dev

int sp24_threads() { return dev::Sp24Cfg::THREADS; }

cudaError_t sp24_launch(const Sp24Args& args, int grid, cudaStream_t stream) {
  static std::atomic<uint64_t> done{0};
  int d = 0;
  if (cudaGetDevice(&d) != cudaSuccess) return cudaErrorInvalidDevice;
  const uint64_t bit = d < 64 ? (1ull << d) : 0;
  if (!bit || !(done.load() & bit)) {
    const cudaError_t e = cudaFuncSetAttribute(dev::spmm24_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                               dev::Sp24Cfg::SMEM_BYTES);
    if (e != cudaSuccess) {
      cudaGetLastError();
      return e;
    }
    done.fetch_or(bit);
  }
  dev::spmm24_kernel<<<grid, dev::Sp24Cfg::THREADS, dev::Sp24Cfg::SMEM_BYTES, stream>>>(args);
  return cudaGetLastError();
}

}  // namespace smat
