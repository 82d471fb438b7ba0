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
// Blocks of a panel are visited in order of their block column, so that the
// B tile of a column is loaded once and used by every block row of the panel
// that has a block there. The A blocks are stored on the device in exactly
// that visiting order, already in the shared-memory layout the MMA reads
// (32-byte swizzle). The pipeline moves STAGES: one stage carries up to 16
// A blocks (8 of 32 rows), up to 8 packed B tiles those blocks need and the
// stage's MMA list (precomputed on the host, stored after the stage's A
// blocks so that one copy brings both), so the hand-off between the copy
// engine and the tensor cores is one full/empty barrier pair per stage.
//
// Roles (512 threads):
//   warps 8..15     copy warps: a stage needs one bulk copy for its A blocks
//                   and list and one per B tile; the copies rotate over the
//                   eight warps (a warp keeps only about one copy at a time
//                   in flight).
//   warps 0..3      MMA issuers, lane 0 each, one per quarter of the panel's
//                   block rows (one thread issues at most one tcgen05.mma
//                   per ~80-150 cycles; four keep the tensor pipe at its
//                   per-instruction rate); warp 0 also owns TMEM.
//   warps 4..7      epilogue: tcgen05.ld -> row scatter through row_map ->
//                   FP32 or FP16 stores of C (coalesced along N).
//
// Consecutive block rows with a block at the same column form one MMA
// (N = bh * run length), so dense panels need far fewer instructions.
//
// Every wait is bounded (see tc_ptx.cuh); on a timeout the kernel raises the
// CTA's abort flag, records the site in the global error word, lets the
// producers wait for their own copies in flight and the MMA threads for
// their own MMAs, frees TMEM and returns.
#include <cuda.h>
#include <cuda_bf16.h>
#include <cuda_fp16.h>
#include <cuda_runtime.h>

#include <atomic>
#include <cstdint>

#include "spmm_tc.h"
#include "tc_ptx.cuh"

namespace smat {
namespace dev {

enum : int { KIND_PLAIN = 0, KIND_SPLIT = 1, KIND_FP8 = 2 };


// Error sites recorded in the global error word.
enum : int {
  ERR_PROD_A = 102,
  ERR_PROD_B = 101,
  ERR_MMA_ACC = 201,
  ERR_MMA_A = 202,
  ERR_MMA_B = 203,
  ERR_MMA_STALL = 205,  // the test stall (SpmmArgs::stall_stage)
  ERR_EPI = 301,
  ERR_CONV = 302,
  ERR_DRAIN = 401,
  ERR_ITEM_TAKE = 103,  // the copy warps waited for a free item-ring slot
  ERR_ITEM_MMA = 204,   // an MMA warp waited for its next item
  ERR_ITEM_EPI = 303,
  ERR_ITEM_CONV = 304
};

// Entries of the CTA's ring of work items (the copy warps take items from
// the launch's counter and run up to a few items ahead of the other roles).
constexpr int kItemRing = 4;

template <int BH, int R, int NSUB, int KIND>
struct Cfg {
  static constexpr int BN = 128 * NSUB;                   // C columns per tile
  static constexpr int NOPS = (KIND == KIND_SPLIT) ? 2 : 1;
  // plan class (stage shape): 256-column B tiles (NSUB 2) halve the tiles per stage
  static constexpr int CLS = KIND == KIND_SPLIT ? 1 : (KIND == KIND_FP8 ? 2 : (NSUB == 2 ? 3 : 0));
  static constexpr int SB = stage_rows(CLS) / BH;         // A blocks per stage (at most)
  static constexpr int ST = stage_tiles(CLS);             // B tiles per stage (at most)
  static constexpr int HDRMAX = stage_hdr_max(SB);
  static constexpr uint32_t ABLK = BH * 32;               // bytes of one A block (one operand)
  static constexpr uint32_t TILE = BN * 32;               // bytes of one B tile (one operand)
  static constexpr uint32_t TILEB = TILE * NOPS;          // bytes of one B tile slot
  static constexpr bool FP8 = KIND == KIND_FP8;
  // stage: [A blocks hi | lo | header] [B tiles] [header offset word]; the
  // FP8 form lands [e4m3 blocks | scales | header] in a staging area after
  // the A blocks, which the converter warps turn into FP16 A blocks
  static constexpr uint32_t OFF_STG = SB * ABLK * NOPS;
  static constexpr uint32_t STG_BYTES = FP8 ? (SB * 256 + fp8_scale_bytes(SB) + HDRMAX + 255) / 256 * 256 : 0;
  static constexpr uint32_t A_END = FP8 ? OFF_STG + STG_BYTES : OFF_STG + HDRMAX;
  static constexpr uint32_t OFF_B = (A_END + 1023) / 1024 * 1024;
  static constexpr uint32_t OFF_HW = OFF_B + ST * TILEB;
  static constexpr uint32_t STAGE = (OFF_HW + 16 + 1023) / 1024 * 1024;
  static constexpr uint32_t SMEM_AVAIL = 227 * 1024 - 2048;  // minus alignment slack and barriers
  static constexpr int NS_FIT = (int)(SMEM_AVAIL / STAGE);
  static constexpr int NS = NS_FIT < 2 ? 2 : (NS_FIT > 8 ? 8 : NS_FIT);  // stages
  static constexpr uint32_t SUB_COLS = R * BH;            // TMEM columns of one 128-column subtile
  static constexpr uint32_t ACC_COLS = NSUB * SUB_COLS;   // TMEM columns per buffer
  static constexpr uint32_t TMEM_COLS = 2 * ACC_COLS;
  static constexpr int NMMA = kMmaWarps;                  // MMA-issuing warps
  static constexpr int NPROD = 8;                         // copy warps
  static constexpr int NCONV = FP8 ? 4 : 0;               // FP8 converter warps (16..19)
  static constexpr uint32_t SMEM_BARS = 8 * (2 * NS + 4 + NMMA + (FP8 ? 2 * NS : 0) + 2 * kItemRing + 1);
  // then the TMEM address, the abort flag, stage_ok[NS], the item ring and
  // the copy warps' current item
  static constexpr uint32_t SMEM_BYTES = 1024 + NS * STAGE + SMEM_BARS + 8 + 4 * (NS + kItemRing + 1);
  static constexpr int THREADS = 32 * (8 + NPROD + NCONV);  // MMA, epilogue, copy, converter warps
  static_assert(TMEM_COLS >= 32 && TMEM_COLS <= 512 && (TMEM_COLS & (TMEM_COLS - 1)) == 0,
                "TMEM allocation must be a power of two in [32, 512]");
  static_assert(BH == 16 || BH == 32, "block height");
  static_assert(NSUB == 1 || (NSUB == 2 && KIND == KIND_PLAIN), "256-column tiles: plain form only");
  static_assert(R <= 32, "slot field is 5 bits");
  static_assert(SB <= kMaxStageBlocks, "position field is 5 bits");
  // a stage tile of NSUB 128-column subtiles is NSUB copies (packed B is
  // [128-column tile][k-block]: the subtiles are not adjacent)
  static_assert(ST * NSUB + 1 <= 2 * NPROD && ST <= kMaxStageTiles,
                "1 + ST * NSUB copies per stage, at most two per copy warp");
  static_assert(NS_FIT >= 2, "two stages must fit");
  static_assert(SMEM_BYTES <= 227 * 1024, "shared memory per CTA");
  static_assert(!FP8 || (BH == 16 && NSUB == 1), "FP8 form: 16 x 16 blocks, 128-column tiles");
};

// Wait used only while draining after an abort: bounded, ignores the flag.
__device__ __noinline__ bool mbar_wait_drain(uint32_t bar, uint32_t parity, int* err, uint64_t lim) {
  const uint64_t t0 = globaltimer();
  while (!mbar_try_wait(bar, parity)) {
    if (globaltimer() - t0 > lim) {
      atomicCAS(err, 0, ERR_DRAIN);
      return false;
    }
  }
  return true;
}

// Bounded wait with an inlined fast path for phases that already completed.
__device__ __forceinline__ bool wait_phase(uint32_t bar, uint32_t parity, volatile int* abort, int* err,
                                           int where, uint64_t lim) {
  return mbar_try_wait(bar, parity) || mbar_wait(bar, parity, abort, err, where, lim);
}

__device__ __forceinline__ bool wait_phase_sleepy(uint32_t bar, uint32_t parity, volatile int* abort, int* err,
                                                  int where, uint64_t lim) {
  return mbar_try_wait(bar, parity) || mbar_wait_sleepy(bar, parity, abort, err, where, lim);
}

// Item k of the CTA from the item ring, for a role run by lane 0 alone:
// waits for it, reads it and frees the ring slot. idx = -1: no more work.
// Returns false when the CTA aborted.
__device__ __forceinline__ bool take_item_lane0(uint64_t* itemfull, uint64_t* itemempty, const volatile int* ring,
                                                uint32_t k, volatile int* abort, int* err, int where, uint64_t lim,
                                                int& idx) {
  const uint32_t r = k % kItemRing;
  if (!wait_phase(smem_u32(&itemfull[r]), (k / kItemRing) & 1, abort, err, where, lim)) return false;
  idx = ring[r];
  mbar_arrive(smem_u32(&itemempty[r]));
  return true;
}

// The same for a whole warp: lane 0 waits and reads, the warp gets the
// index by shuffle (so the warp's decision is uniform).
__device__ __forceinline__ bool take_item_warp(uint64_t* itemfull, uint64_t* itemempty, const volatile int* ring,
                                               uint32_t k, int lane, volatile int* abort, int* err, int where,
                                               uint64_t lim, int& idx) {
  int got = 1, v = -1;
  if (lane == 0) {
    const uint32_t r = k % kItemRing;
    got = wait_phase_sleepy(smem_u32(&itemfull[r]), (k / kItemRing) & 1, abort, err, where, lim) ? 1 : 0;
    if (got) {
      v = ring[r];
      mbar_arrive(smem_u32(&itemempty[r]));
    }
  }
  got = __shfl_sync(0xffffffffu, got, 0);
  idx = __shfl_sync(0xffffffffu, v, 0);
  return got != 0;
}

// The copy index that copy warp pw issues first in stage c: copy j of a
// stage goes to warp (j + c) mod nprod, so the duties rotate.
__device__ __forceinline__ int copy_of(int pw, uint32_t c, int nprod) {
  return (int)(((uint32_t)pw + (uint32_t)nprod - c % (uint32_t)nprod) % (uint32_t)nprod);
}

// Bounded wait for a whole warp: lane 0 polls, the warp learns the outcome
// by shuffle and leaves converged (lanes that each polled would leave the
// loop on different iterations and could run the code after it diverged).
__device__ __forceinline__ bool warp_wait(uint32_t bar, uint32_t parity, int lane, volatile int* abort, int* err,
                                          int where, bool sleepy, uint64_t lim) {
  int got = 1;
  if (lane == 0)
    got = (sleepy ? wait_phase_sleepy(bar, parity, abort, err, where, lim)
                  : wait_phase(bar, parity, abort, err, where, lim))
              ? 1
              : 0;
  return __shfl_sync(0xffffffffu, got, 0) != 0;
}

__device__ __forceinline__ int shfl_i(int v, int src) { return __shfl_sync(0xffffffffu, v, src); }
__device__ __forceinline__ int64_t shfl_l(int64_t v, int src) {
  const int lo = __shfl_sync(0xffffffffu, (int)(uint32_t)(uint64_t)v, src);
  const int hi = __shfl_sync(0xffffffffu, (int)(uint32_t)((uint64_t)v >> 32), src);
  return (int64_t)(((uint64_t)(uint32_t)hi << 32) | (uint32_t)lo);
}

// Warp roles: 0..3 MMA issuers (0 also owns TMEM), 4..7 epilogue (TMEM lane
// quadrants 0..3), then NPROD copy warps, then (FP8) the converter warps.
template <int BH, int R, int NSUB, int KIND>
__global__ void __launch_bounds__(Cfg<BH, R, NSUB, KIND>::THREADS, 1)
    spmm_tc_kernel(const __grid_constant__ SpmmArgs args) {
  using C = Cfg<BH, R, NSUB, KIND>;
  extern __shared__ uint8_t smem_raw[];
  uint8_t* smem = reinterpret_cast<uint8_t*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) &
                                             ~static_cast<uintptr_t>(1023));
  uint64_t* bars = reinterpret_cast<uint64_t*>(smem + C::NS * C::STAGE);
  uint64_t* full = bars;
  uint64_t* empty = full + C::NS;
  uint64_t* accfull = empty + C::NS;
  uint64_t* accempty = accfull + 2;
  uint64_t* drainbar = accempty + 2;
  uint64_t* conv = drainbar + C::NMMA;  // FP8: the stage's A blocks are converted
  // FP8: the stage's A copy landed (the converters start on it while the B
  // tiles are still landing on full[])
  uint64_t* afull = conv + (C::FP8 ? C::NS : 0);
  uint64_t* itemfull = afull + (C::FP8 ? C::NS : 0);  // [kItemRing] an item index is in the ring
  uint64_t* itemempty = itemfull + kItemRing;        // [kItemRing] every role has read it
  uint64_t* stallbar = itemempty + kItemRing;        // nothing arrives here (test stall)
  uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(stallbar + 1);
  volatile int* abort_flag = reinterpret_cast<volatile int*>(tmem_slot + 1);
  volatile int* stage_ok = abort_flag + 1;  // [NS]: the copy leader's verdict on the stage's slot
  volatile int* item_ring = stage_ok + C::NS;     // [kItemRing] item indices (-1: no more work)
  volatile int* cur_item = item_ring + kItemRing;  // the copy warps' current item

  const int warp = threadIdx.x >> 5;
  const int lane = threadIdx.x & 31;
  const uint64_t lim = args.wait_ns ? args.wait_ns : kWaitTimeoutNs;
  // stage slots in use (the pipeline depth): all that fit, or fewer when the
  // launch asks
  const uint32_t nsr = (args.depth >= 2 && args.depth < C::NS) ? (uint32_t)args.depth : (uint32_t)C::NS;

  if (threadIdx.x == 0) {
    for (int i = 0; i < C::NS; i++) {
      mbar_init(smem_u32(&full[i]), 1);  // the A copy warp's arrive (+ every copy's bytes)
      mbar_init(smem_u32(&empty[i]), C::NMMA);
    }
    for (int i = 0; i < 2; i++) {
      mbar_init(smem_u32(&accfull[i]), C::NMMA);
      mbar_init(smem_u32(&accempty[i]), 4);
    }
    for (int i = 0; i < C::NMMA; i++) mbar_init(smem_u32(&drainbar[i]), 1);
    if (C::FP8)
      for (int i = 0; i < C::NS; i++) {
        mbar_init(smem_u32(&conv[i]), C::NCONV);
        mbar_init(smem_u32(&afull[i]), 1);
      }
    for (int i = 0; i < kItemRing; i++) {
      mbar_init(smem_u32(&itemfull[i]), 1);
      mbar_init(smem_u32(&itemempty[i]), C::NMMA + 4 + C::NCONV);  // lane 0 of every other warp
    }
    mbar_init(smem_u32(stallbar), 1);
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

  int* err = args.err;
  const uint32_t smem0 = smem_u32(smem);

  if (C::FP8 && warp >= 8 + C::NPROD) {
    // ------------------------------------------------------ FP8 converters
    // Each stage's e4m3 blocks and FP32 scales land in the staging area;
    // these four warps write them to the stage's A area as FP16 (value times
    // its block's scale, one rounding) in the 32-byte-swizzled layout the
    // MMA reads, make the writes visible to the tensor core's async proxy,
    // and release the stage to the MMA warps (conv barrier).
    const int ct = threadIdx.x - 32 * (8 + C::NPROD);
    uint32_t ci = 0;
    bool ok = true;
    for (uint32_t kk = 0; ok; ++kk) {
      int idx = -1;
      if (!take_item_warp(itemfull, itemempty, item_ring, kk, lane, abort_flag, err, ERR_ITEM_CONV, lim, idx)) {
        ok = false;
        break;
      }
      if (idx < 0) break;
      const WorkItem wi = args.items[idx];
      const ProblemDesc& P = args.probs ? args.probs[wi.prob] : args.one;
      const int n_tiles = P.n_tiles;
      for (int nt = 0; nt < n_tiles && ok; ++nt) {
        for (int c = wi.s0; c < wi.s1; ++c, ++ci) {
          const uint32_t s = ci % nsr;
          if (!warp_wait(smem_u32(&afull[s]), (ci / nsr) & 1, lane, abort_flag, err, ERR_CONV, false, lim)) {
            ok = false;
            break;
          }
          uint8_t* stp = smem + s * C::STAGE;
          const uint32_t hw = *reinterpret_cast<const uint32_t*>(stp + C::OFF_HW);
          const int nblk = *reinterpret_cast<const uint16_t*>(stp + hw + 8);
          const uint8_t* stg = stp + C::OFF_STG;
          const float* scl = reinterpret_cast<const float*>(stg + nblk * 256);
          for (int x = ct; x < nblk * 32; x += 128) {
            const int b = x >> 5, r = (x >> 1) & 15, hh = x & 1;  // block, row, 8-column half
            const uint2 raw = *reinterpret_cast<const uint2*>(stg + b * 256 + r * 16 + hh * 8);
            const float sc = scl[b];
            uint32_t w[4];
#pragma unroll
            for (int i = 0; i < 4; ++i) {
              const uint16_t pair = (uint16_t)(((i < 2 ? raw.x : raw.y) >> (16 * (i & 1))) & 0xffffu);
              const float2 f = __half22float2(e4m3x2_to_half2(pair));
              const __half2 o = __floats2half2_rn(f.x * sc, f.y * sc);
              w[i] = *reinterpret_cast<const uint32_t*>(&o);
            }
            *reinterpret_cast<uint4*>(stp + b * 512 + r * 32 + ((hh ^ ((r >> 2) & 1)) << 4)) =
                make_uint4(w[0], w[1], w[2], w[3]);
          }
          fence_proxy_async_smem();
          __syncwarp();
          if (lane == 0) mbar_arrive(smem_u32(&conv[s]));
        }
      }
    }
  } else if (warp >= 8) {
    // ---------------------------------------------------------------- copies
    // Stage number c (counted over the CTA's whole run) needs 1 + ntiles
    // bulk copies: copy 0 = the A blocks and the MMA list, copy j = B tile
    // j - 1. Copy warp p issues the copies j with (j + c) % NPROD == p (j and
    // j + NPROD), so every warp issues one or two copies per stage and the A
    // copy (from HBM, the slowest) rotates. A warp keeps only about one copy
    // at a time in flight, so spreading them is what keeps the copy engine
    // busy. The warp that
    // issues copy 0 posts the stage's total byte count (arrive.expect_tx) on
    // the stage's full barrier; the others only add their bytes as they land.
    // Stage records are read 32 at a time, one per lane, and each lane
    // prepares what its warp needs from its record.
    const int pw = warp - 8;
    const uint64_t pol_a = make_l2_policy_evict_first();  // A streams through L2 once
    const uint64_t pol_b = make_l2_policy_evict_last();   // B tiles are re-read by many CTAs
    uint32_t ci = 0;
    bool ok = true;
    uint32_t last_mine = 0xffffffffu;  // last stage this warp copied into (for the drain)
    for (uint32_t kk = 0; ok; ++kk) {
      // The CTA's next item: lane 0 of the first copy warp takes it from the
      // launch's order (the CTA's own index first, then the shared
      // counter), puts it in the item ring for the other roles once they
      // have read the entry it replaces, and hands it to the copy warps.
      if (pw == 0 && lane == 0) {
        const uint32_t r = kk % kItemRing;
        int idx = -2;  // -2: aborted
        if (wait_phase(smem_u32(&itemempty[r]), ((kk / kItemRing) & 1) ^ 1, abort_flag, err, ERR_ITEM_TAKE, lim)) {
          const int pos = kk == 0 ? (int)blockIdx.x : (int)gridDim.x + atomicAdd(args.next_item, 1);
          idx = pos < args.n_items ? args.order[pos] : -1;
          item_ring[r] = idx;
          mbar_arrive(smem_u32(&itemfull[r]));
        }
        *cur_item = idx;
      }
      named_bar_sync(1, 32 * C::NPROD);
      const int idx = *cur_item;
      if (idx < 0) {
        ok = idx == -1;
        break;
      }
      const WorkItem wi = args.items[idx];
      const ProblemDesc& P = args.probs ? args.probs[wi.prob] : args.one;
      // fields used after shared-memory stores, held in registers (the stores
      // could alias P for the compiler and force a reload each time)
      const StageRec* const p_stages = P.stages;
      const uint8_t* const p_aval = P.aval;
      const uint8_t* const p_bpack = P.bpack;
      const int64_t p_kbs = P.bp_kbs;
      const int n_tiles = P.n_tiles;
      const int stage0 = P.panels[wi.panel].stage_off;
      for (int nt = 0; nt < n_tiles && ok; ++nt) {
        const int64_t bcol = (int64_t)nt * NSUB;  // first 128-column packed tile of this pass
        for (int base = wi.s0; base < wi.s1 && ok; base += 32) {
          const int cnt = min(32, wi.s1 - base);
          // lane l prepares stage ci + l
          const uint32_t my_ci = ci + (uint32_t)lane;
          const int j0 = copy_of(pw, my_ci, C::NPROD);
          int64_t off1 = 0, off2 = 0;
          int bytes1 = 0, bytes2 = 0, dst1 = 0, dst2 = 0, total = 0, hword = 0;
          if (lane < cnt) {
            const StageRec* rp = p_stages + stage0 + base + lane;
            const longlong2 r0 = reinterpret_cast<const longlong2*>(rp)[0];  // blk_off, hdr_off
            const int4 r1 = reinterpret_cast<const int4*>(rp)[1];           // nblk, hdr_bytes, ntiles, -
            const int ntl = r1.z;
            if (j0 == 0) {
              // the stage's A region (blocks, FP8 scales, header) in one copy
              // (an L2 prefetch of it a few stages ahead measured slower:
              // it competes with the copies for the copy engine)
              if (C::FP8) {
                off1 = r0.x * 256 + r1.w + r0.y;
                bytes1 = r1.x * 256 + fp8_scale_bytes(r1.x) + r1.y;
              } else {
                off1 = r0.x * (int64_t)(C::ABLK * C::NOPS) + r0.y;
                bytes1 = r1.x * (int)(C::ABLK * C::NOPS) + r1.y;
              }
              // header position inside the stage
              hword = C::FP8 ? (int)C::OFF_STG + r1.x * 256 + fp8_scale_bytes(r1.x) : r1.x * (int)(C::ABLK * C::NOPS);
              total = bytes1 + ntl * (int)C::TILEB;
            }
            // B copies, one per 128-column subtile (several copies in flight
            // land sooner than one long copy of adjacent tiles): copy c >= 1
            // brings subtile (c - 1) % NSUB of tile (c - 1) / NSUB; this
            // warp's are copies j0 and j0 + NPROD
            if (j0 >= 1 && j0 <= ntl * NSUB) {
              const int t = (j0 - 1) / NSUB, sub = (j0 - 1) % NSUB;
              off1 = ((int64_t)(bcol + sub) * p_kbs + rp->kb[t]) * (4096 * C::NOPS);
              bytes1 = 4096 * C::NOPS;
              dst1 = t * (int)C::TILEB + sub * 4096 * C::NOPS;
            }
            if (j0 + C::NPROD <= ntl * NSUB) {
              const int t = (j0 + C::NPROD - 1) / NSUB, sub = (j0 + C::NPROD - 1) % NSUB;
              off2 = ((int64_t)(bcol + sub) * p_kbs + rp->kb[t]) * (4096 * C::NOPS);
              bytes2 = 4096 * C::NOPS;
              dst2 = t * (int)C::TILEB + sub * 4096 * C::NOPS;
            }
          }
          for (int i = 0; i < cnt; ++i, ++ci) {
            const int b1 = shfl_i(bytes1, i);
            const int b2 = shfl_i(bytes2, i);
            const int d1 = shfl_i(dst1, i);
            const int d2 = shfl_i(dst2, i);
            const int64_t o1 = shfl_l(off1, i);
            const int64_t o2 = shfl_l(off2, i);
            const int tot = shfl_i(total, i);
            const int hw = shfl_i(hword, i);
            const int j = copy_of(pw, ci, C::NPROD);
            const uint32_t s = ci % nsr;
            // The warp with copy 0 waits for the slot and passes its verdict
            // to the other copy warps through a named barrier (blocked warps
            // take no issue slots); so all copy warps move stage by stage and
            // none can run a ring ahead and overwrite a stage still in use.
            if (j == 0 && lane == 0)
              stage_ok[s] = wait_phase(smem_u32(&empty[s]), ((ci / nsr) & 1) ^ 1, abort_flag, err, ERR_PROD_A, lim) ? 1 : 0;
            named_bar_sync(1, 32 * C::NPROD);
            int good = 1;
            if (lane == 0) {
              if (stage_ok[s]) {
                const uint32_t st = smem0 + s * C::STAGE;
                const uint32_t fb = smem_u32(&full[s]);
                if (b1 == 0) {
                  // no copy for this warp in this stage
                } else if (j == 0) {
                  *reinterpret_cast<uint32_t*>(smem + s * C::STAGE + C::OFF_HW) = (uint32_t)hw;
                  if (C::FP8) {
                    // the A region on its own barrier (the converters wait
                    // for it alone), the B tiles on full[s]
                    const uint32_t ab = smem_u32(&afull[s]);
                    mbar_arrive_expect_tx(ab, (uint32_t)b1);
                    bulk_load_hint(st + C::OFF_STG, p_aval + o1, (uint32_t)b1, ab, pol_a);
                    mbar_arrive_expect_tx(fb, (uint32_t)(tot - b1));
                  } else {
                    mbar_arrive_expect_tx(fb, (uint32_t)tot);
                    bulk_load_hint(st, p_aval + o1, (uint32_t)b1, fb, pol_a);
                  }
                } else {
                  bulk_load_hint(st + C::OFF_B + d1, p_bpack + o1, (uint32_t)b1, fb, pol_b);
                }
                if (b2 != 0) bulk_load_hint(st + C::OFF_B + d2, p_bpack + o2, (uint32_t)b2, fb, pol_b);
                if (b1 != 0 || b2 != 0) last_mine = ci;
              } else {
                good = 0;
              }
            }
            good = shfl_i(good, 0);
            if (!good) {
              ok = false;
              break;
            }
          }
        }
      }
    }
    if (!ok && lane == 0 && last_mine != 0xffffffffu) {
      // wait for this warp's own copies still in flight: they can only be in
      // the last NS stages it copied into
      const uint32_t lo = last_mine + 1 > nsr ? last_mine + 1 - nsr : 0;
      for (uint32_t k = lo; k <= last_mine; ++k) {
        mbar_wait_drain(smem_u32(&full[k % nsr]), (k / nsr) & 1, err, lim);
        if (C::FP8) mbar_wait_drain(smem_u32(&afull[k % nsr]), (k / nsr) & 1, err, lim);
      }
    }
  } else if (warp < C::NMMA) {
    if (lane == 0) {
      // ----------------------------------------------------------- MMA issuers
      // Issuer w runs the MMA groups of its quarter of the panel's block rows,
      // from the list the copy brought in with the stage, and releases every
      // stage once. One thread issues a tcgen05.mma only every ~80-150
      // cycles; four keep the tensor pipe near its rate for these narrow MMAs.
      uint32_t ci = 0, k = 0, slot_s = 0, phase_s = 0;
      bool ok = true, issued = false;
      const uint32_t stall = (blockIdx.x == 0 && warp == 0) ? (uint32_t)args.stall_stage : 0u;
      for (uint32_t kk = 0; ok; ++kk) {
        int idx = -1;
        if (!take_item_lane0(itemfull, itemempty, item_ring, kk, abort_flag, err, ERR_ITEM_MMA, lim, idx)) {
          ok = false;
          break;
        }
        if (idx < 0) break;
        const WorkItem wi = args.items[idx];
        const ProblemDesc& P = args.probs ? args.probs[wi.prob] : args.one;
        const int n_tiles = P.n_tiles;
        const uint32_t idesc0 = P.idesc;  // without the N field
        const int nstages = wi.s1 - wi.s0;
        for (int nt = 0; nt < n_tiles && ok; ++nt, ++k) {
          const uint32_t buf = k & 1;
          const uint32_t dbase = tmem + buf * C::ACC_COLS;
          // use u = k / 2 of this buffer waits for phase u of accempty: the
          // epilogue's initial zeroing (u = 0), then each drain-and-zero
          if (!wait_phase(smem_u32(&accempty[buf]), (k >> 1) & 1, abort_flag, err, ERR_MMA_ACC, lim)) {
            ok = false;
            break;
          }
          tc_fence_after();
          for (int c = 0; c < nstages; ++c, ++ci) {
            const uint32_t s = slot_s;  // == ci % nsr, kept incrementally
            if (stall != 0u && ci + 1 == stall) {
              // test stall: nothing arrives on this barrier, so the wait runs
              // into its limit and the CTA aborts
              ok = wait_phase(smem_u32(stallbar), 0, abort_flag, err, ERR_MMA_STALL, lim);
              if (!ok) break;
            }
            // the stage's copies landed (complete_tx); the MMA reads shared
            // memory through the async proxy, so no tcgen05 fence is needed
            // (FP8: the converted A blocks, then the B tiles)
            if (!wait_phase(smem_u32(C::FP8 ? &conv[s] : &full[s]), phase_s, abort_flag, err, ERR_MMA_A, lim) ||
                (C::FP8 && !wait_phase(smem_u32(&full[s]), phase_s, abort_flag, err, ERR_MMA_B, lim))) {
              ok = false;
              break;
            }
            const uint8_t* stp = smem + s * C::STAGE;
            const uint32_t hw = *reinterpret_cast<const uint32_t*>(stp + C::OFF_HW);
            const uint32_t wl = *reinterpret_cast<const uint16_t*>(stp + hw + 2 * warp);
            const uint32_t first = wl & 0xffu, cnt = wl >> 8;
            const uint32_t* ent = reinterpret_cast<const uint32_t*>(stp + hw + kStageHdrFixed) + first;
            // descriptors of operands inside the stage = stage descriptor + offset / 16
            const uint64_t sdesc = desc_kmajor_sw32(smem0 + s * C::STAGE);
            for (uint32_t e = 0; e < cnt; ++e) {
              const uint32_t m = ent[e];
              const uint32_t pos = m & 31u, tile = (m >> 5) & 15u, slot = (m >> 9) & 31u;
              const uint32_t len = ((m >> 14) & 15u) + 1u, acc = (m >> 18) & 1u;
              const uint32_t idesc = idesc0 | (((len * BH) >> 3) << 17);
              const uint64_t a_hi = sdesc + ((pos * C::ABLK) >> 4);
              const uint64_t b_hi0 = sdesc + ((C::OFF_B + tile * C::TILEB) >> 4);
#pragma unroll
              for (int j = 0; j < NSUB; ++j) {
                const uint32_t dcol = dbase + j * C::SUB_COLS + slot * BH;
                const uint64_t b_hi = b_hi0 + ((j * 128 * 32) >> 4);
                umma_f16(dcol, b_hi, a_hi, idesc, acc);
                if (KIND == KIND_SPLIT) {
                  const uint64_t a_lo = a_hi + ((hw >> 1) >> 4);  // lo blocks follow the nblk hi blocks
                  const uint64_t b_lo = b_hi + (C::TILE >> 4);
                  umma_f16(dcol, b_hi, a_lo, idesc, 1);
                  umma_f16(dcol, b_lo, a_hi, idesc, 1);
                }
              }
              issued = true;
            }
            umma_commit(smem_u32(&empty[s]));
            if (++slot_s == nsr) {
              slot_s = 0;
              phase_s ^= 1u;
            }
          }
          if (!ok) break;
          umma_commit(smem_u32(&accfull[buf]));
        }
      }
      if (!ok && issued) {
        const uint32_t db = smem_u32(&drainbar[warp]);
        umma_commit(db);
        mbar_wait_drain(db, 0, err, lim);
      }
    }
  } else if (warp >= 4) {
    // -------------------------------------------------------------- epilogue
    // Warp 4 + q drains TMEM lane quadrant q (C columns q*32 .. q*32+31 of
    // each 128-column subtile) for every slot, and writes zeros back: the
    // accumulators are all zero whenever the MMA warps receive a buffer, so
    // a part that starts in the middle of a panel accumulates onto zero.
    const uint32_t q = warp & 3;
    const uint32_t lane_base = tmem + ((q * 32u) << 16);
    for (uint32_t c = 0; c < 2 * C::ACC_COLS; c += 16) tmem_st_x16_zero(lane_base + c);
    tmem_st_wait();
    tc_fence_before();
    __syncwarp();
    if (lane == 0) {
      mbar_arrive(smem_u32(&accempty[0]));
      mbar_arrive(smem_u32(&accempty[1]));
    }
    constexpr int SLAB = R * BH * C::BN;  // floats per slab
    constexpr int PW = (R % kMmaWarps == 0) ? R / kMmaWarps : 0;  // slots per issuing warp
    constexpr int RPL = (R * BH + 31) / 32;                          // C-row entries per lane
    // 16-row blocks with at least two slots per issuing warp: the drain reads
    // two adjacent slots with one 32-column load (one load round trip per
    // pair; a hub row's later parts are never in their first part's pair).
    // Not for FP8: its 640-thread CTAs have 96 registers a thread, and the
    // pair's 32 values would spill.
    constexpr bool PAIR = BH == 16 && NSUB == 1 && PW >= 2 && R % 2 == 0 && KIND != KIND_FP8;
    uint32_t k = 0;
    bool ok = true;
    for (uint32_t kk = 0; ok; ++kk) {
      int idx = -1;
      if (!take_item_warp(itemfull, itemempty, item_ring, kk, lane, abort_flag, err, ERR_ITEM_EPI, lim, idx)) {
        ok = false;
        break;
      }
      if (idx < 0) break;
      const WorkItem wi = args.items[idx];
      const ProblemDesc& P = args.probs ? args.probs[wi.prob] : args.one;
      // fields used between the stores to C, held in registers (the stores
      // could alias P for the compiler and force reloads of every field)
      const int p_N = P.N, p_nbr = P.nbr, p_f16 = P.c_f16;
      const int64_t p_ldc = P.ldc;
      void* const p_C = P.C;
      float* const p_slabs = P.slabs;
      int32_t* const p_counters = P.counters;
      const int n_tiles = P.n_tiles;
      const int panel = wi.panel;
      const bool split = wi.split >= 0;
      const uint32_t slot_mask = P.panels[panel].slot_mask;
      // a hub row cut over the issuing warps has its parts in slots s, s + PW,
      // s + 2 PW, ...; the parts after the first are added into it here
      const uint32_t ext_mask = P.panels[panel].ext_mask;
      // the panel's C rows, plan row 32 q + lane in rmap[q] of that lane,
      // loaded before the accumulators are ready: one global round trip
      // per item instead of one per slot (the slot loops are unrolled, so
      // rmap stays in registers)
      int rmap[RPL];
#pragma unroll
      for (int q2 = 0; q2 < RPL; ++q2) {
        const int pr = q2 * 32 + lane;
        rmap[q2] = (pr < R * BH && (int64_t)panel * R * BH + pr < (int64_t)p_nbr * BH)
                       ? P.row_map[(int64_t)panel * R * BH + pr]
                       : -1;
      }
      for (int nt = 0; nt < n_tiles; ++nt, ++k) {
        const uint32_t buf = k & 1;
        if (!warp_wait(smem_u32(&accfull[buf]), (k >> 1) & 1, lane, abort_flag, err, ERR_EPI, true, lim)) {
          ok = false;
          break;
        }
        tc_fence_after();
        const uint32_t dbase = lane_base + buf * C::ACC_COLS;
        // slab of (part, column tile): (first slab of the panel + part) * n_tiles + nt
        float* slab = split ? p_slabs + ((size_t)(wi.slab + wi.part) * n_tiles + nt) * SLAB : nullptr;
        float pairv[32];
#pragma unroll
        for (int s = 0; s < R; ++s) {
          const int rb = panel * R + s;
          if (rb >= p_nbr) break;
          if constexpr (PAIR) {
            if ((s & 1) == 0) {
              // slots s and s + 1 (an empty slot reads zeros: slots are
              // zeroed after every drain and no MMA writes an empty one)
              if ((slot_mask >> s) & 3u) {
                const uint32_t ta = dbase + s * BH;
                tmem_ld_x32(ta, pairv);
                tmem_st_x32_zero(ta);
              } else {
#pragma unroll
                for (int m = 0; m < 32; ++m) pairv[m] = 0.0f;
              }
            }
          }
          if ((ext_mask >> s) & 1u) continue;
          const bool empty_slot = ((slot_mask >> s) & 1u) == 0;
#pragma unroll
          for (int j = 0; j < NSUB; ++j) {
            const int nl = j * 128 + (int)q * 32 + lane;  // column inside the tile
            const int n = nt * C::BN + nl;
#pragma unroll
            for (int h = 0; h < BH; h += 16) {
              float vs[16];
              float* v = PAIR ? pairv + (s & 1) * 16 : vs;
              if constexpr (!PAIR) {
                if (!empty_slot) {
                  const uint32_t ta = dbase + j * C::SUB_COLS + s * BH + h;
                  tmem_ld_x16(ta, vs);
                  tmem_st_x16_zero(ta);
                } else {
#pragma unroll
                  for (int m = 0; m < 16; ++m) vs[m] = 0.0f;
                }
              }
              if constexpr (PW > 0) {
                for (int t = s + PW; t < R && ((ext_mask >> t) & 1u); t += PW) {
                  if (((slot_mask >> t) & 1u) == 0) continue;
                  float u[16];
                  const uint32_t tb = dbase + j * C::SUB_COLS + t * BH + h;
                  tmem_ld_x16(tb, u);
                  tmem_st_x16_zero(tb);
#pragma unroll
                  for (int m = 0; m < 16; ++m) v[m] += u[m];
                }
              }
              if (split) {
#pragma unroll
                for (int m = 0; m < 16; ++m) __stcg(slab + (size_t)(s * BH + h + m) * C::BN + nl, v[m]);
              } else {
#pragma unroll
                for (int m = 0; m < 16; ++m) {
                  const int pr = s * BH + h + m;  // plan row inside the panel
                  const int row = __shfl_sync(0xffffffffu, rmap[pr >> 5], pr & 31);
                  if (row >= 0 && n < p_N) {
                    const int64_t off = (int64_t)row * p_ldc + n;
                    if (p_f16)
                      __stcs(reinterpret_cast<__half*>(p_C) + off, __float2half_rn(v[m]));
                    else
                      __stcs(reinterpret_cast<float*>(p_C) + off, v[m]);
                  }
                }
              }
            }
          }
        }
        tmem_st_wait();
        tc_fence_before();
        __syncwarp();
        if (lane == 0) mbar_arrive(smem_u32(&accempty[buf]));
        if (!split) continue;
        // this warp's part of the slab is written: count it; the warp that
        // brings the count of its quadrant to nparts adds up all parts
        __threadfence();
        __syncwarp();
        int last = 0;
        if (lane == 0) {
          int* ctr = p_counters + ((size_t)wi.split * n_tiles + nt) * 4 + q;
          last = atomicAdd(ctr, 1) == wi.nparts - 1;
        }
        last = __shfl_sync(0xffffffffu, last, 0);
        if (!last) continue;
        __threadfence();
        const float* slab0 = p_slabs + ((size_t)wi.slab * n_tiles + nt) * SLAB;
#pragma unroll
        for (int s = 0; s < R; ++s) {
          const int rb = panel * R + s;
          if (rb >= p_nbr) break;
          if ((ext_mask >> s) & 1u) continue;  // added into its first part's slab rows
#pragma unroll
          for (int j = 0; j < NSUB; ++j) {
            const int nl = j * 128 + (int)q * 32 + lane;
            const int n = nt * C::BN + nl;
            for (int h = 0; h < BH; h += 16) {
              // 16 rows at a time: the loads of a part are independent, so
              // they overlap instead of paying one L2 round trip per row
              float acc[16];
#pragma unroll
              for (int m = 0; m < 16; ++m) acc[m] = 0.0f;
              const float* src = slab0 + (size_t)(s * BH + h) * C::BN + nl;
              for (int p = 0; p < wi.nparts; ++p) {
                float t[16];
#pragma unroll
                for (int m = 0; m < 16; ++m) t[m] = __ldcg(src + (size_t)m * C::BN);
#pragma unroll
                for (int m = 0; m < 16; ++m) acc[m] += t[m];
                src += (size_t)n_tiles * SLAB;
              }
#pragma unroll
              for (int m = 0; m < 16; ++m) {
                const int pr = s * BH + h + m;
                const int row = __shfl_sync(0xffffffffu, rmap[pr >> 5], pr & 31);
                if (row >= 0 && n < p_N) {
                  const int64_t off = (int64_t)row * p_ldc + n;
                  if (p_f16)
                    __stcs(reinterpret_cast<__half*>(p_C) + off, __float2half_rn(acc[m]));
                  else
                    __stcs(reinterpret_cast<float*>(p_C) + off, acc[m]);
                }
              }
            }
          }
        }
      }
    }
  }

  // lane 0 of the MMA and copy warps ran their roles alone: reconverge
  // every warp before the CTA-wide barrier
  __syncwarp();
  tc_fence_before();
  __syncthreads();
  if (warp == 0) {
    tc_fence_after();
    tmem_dealloc(tmem, C::TMEM_COLS);
  }
}

// Raises the variant's dynamic shared memory limit once per device (a
// launch inside a stream capture then makes no other CUDA call).
template <int BH, int R, int NSUB, int KIND>
static cudaError_t prepare_one() {
  using C = Cfg<BH, R, NSUB, KIND>;
  static std::atomic<uint64_t> done{0};
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return cudaErrorInvalidDevice;
  const uint64_t bit = dev < 64 ? (1ull << dev) : 0;
  if (bit && (done.load() & bit)) return cudaSuccess;
  const cudaError_t e = cudaFuncSetAttribute(spmm_tc_kernel<BH, R, NSUB, KIND>,
                                             cudaFuncAttributeMaxDynamicSharedMemorySize, C::SMEM_BYTES);
  if (e != cudaSuccess) {
    cudaGetLastError();  // do not leave the error for the next call to find
    return e;
  }
  done.fetch_or(bit);
  return cudaSuccess;
}

template <int BH, int R, int NSUB, int KIND>
static cudaError_t launch_one(const SpmmArgs& args, int grid, cudaStream_t stream) {
  using C = Cfg<BH, R, NSUB, KIND>;
  auto kfn = spmm_tc_kernel<BH, R, NSUB, KIND>;
  cudaError_t e = prepare_one<BH, R, NSUB, KIND>();
  if (e != cudaSuccess) return e;
  kfn<<<grid, C::THREADS, C::SMEM_BYTES, stream>>>(args);
  return cudaGetLastError();
}

// Co-resident CTAs per SM: limited by TMEM (512 columns per SM) and by what
// the occupancy calculator reports for the shared memory and registers.
template <int BH, int R, int NSUB, int KIND>
static int ctas_per_sm_one() {
  using C = Cfg<BH, R, NSUB, KIND>;
  auto kfn = spmm_tc_kernel<BH, R, NSUB, KIND>;
  int by_tmem = 512 / C::TMEM_COLS;
  int occ = 1;
  if (prepare_one<BH, R, NSUB, KIND>() != cudaSuccess ||
      cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, kfn, C::THREADS, C::SMEM_BYTES) != cudaSuccess) {
    cudaGetLastError();
    occ = 1;
  }
  int n = by_tmem < occ ? by_tmem : occ;
  return n < 1 ? 1 : n;
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
  X(16, 4, 1, 1)            \
  X(16, 8, 1, 1)            \
  X(16, 16, 1, 1)           \
  X(32, 4, 1, 1)            \
  X(32, 8, 1, 1)            \
  X(16, 4, 1, 2)            \
  X(16, 8, 1, 2)            \
  X(16, 16, 1, 2)

bool tc_variant_supported(int bh, int R, int nsub, int kind) {
#define SMAT_TC_MATCH(BH, R_, NS, K) \
  if (bh == BH && R == R_ && nsub == NS && kind == K) return true;
  SMAT_TC_VARIANTS(SMAT_TC_MATCH)
#undef SMAT_TC_MATCH
  return false;
}

int tc_ctas_per_sm(int bh, int R, int nsub, int kind) {
#define SMAT_TC_OCC(BH, R_, NS, K) \
  if (bh == BH && R == R_ && nsub == NS && kind == K) return dev::ctas_per_sm_one<BH, R_, NS, K>();
  SMAT_TC_VARIANTS(SMAT_TC_OCC)
#undef SMAT_TC_OCC
  return 1;
}

cudaError_t tc_launch(int bh, int R, int nsub, int kind, const SpmmArgs& args, int grid,
                      cudaStream_t stream) {
#define SMAT_TC_LAUNCH(BH, R_, NS, K)                             \
  if (bh == BH && R == R_ && nsub == NS && kind == K) \
    return dev::launch_one<BH, R_, NS, K>(args, grid, stream);
  SMAT_TC_VARIANTS(SMAT_TC_LAUNCH)
#undef SMAT_TC_LAUNCH
  return cudaErrorInvalidValue;
}

}  // namespace smat
