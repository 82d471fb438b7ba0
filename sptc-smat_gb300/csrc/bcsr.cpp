// bcsr.cpp — CSR -> BCSR on the host, and the tensor-core work plan.
//
// The block structure is bit-identical to SparseMatrix::csrToBcsr
// (src/cuda_hgemm/src/common/matrix.h:666-792): per block row the nonzero
// block columns in ascending order, bcsrColIdx = the column START of the
// block, values row-major inside a block, zero-filled, the last CSR entry of
// a duplicated (row, col) winning. Unlike the reference it does not allocate
// the dense (rows/bh) x (cols/bw) block grid (1 GiB per array for a 256K x
// 256K matrix); it works block row by block row with a stamp array.
#include <omp.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <numeric>

#include "fp_convert.h"
#include "smat_internal.h"

namespace smat {

smat_status build_host_bcsr(const smat_csr& A, int32_t bh, int32_t bw, const int64_t* perm,
                            HostBcsr& out) {
  if (A.rows < 0 || A.cols < 0 || A.nnz < 0) return fail(SMAT_ERR_INVALID, "negative CSR size");
  if (!A.row_ptr || (A.nnz > 0 && !A.col_idx)) return fail(SMAT_ERR_INVALID, "CSR arrays missing");
  if (A.values && A.values_dtype != SMAT_F32 && A.values_dtype != SMAT_F16 &&
      A.values_dtype != SMAT_F64)
    return fail(SMAT_ERR_INVALID, "CSR values must be F32, F16 or F64");
  if (!(bh == 8 || bh == 16 || bh == 32) || !(bw == 8 || bw == 16 || bw == 32))
    return fail(SMAT_ERR_UNSUPPORTED, "block shape must be 8, 16 or 32 on each side");
  if (A.row_ptr[0] != 0 || A.row_ptr[A.rows] != A.nnz)
    return fail(SMAT_ERR_INVALID, "row_ptr[0] must be 0 and row_ptr[rows] == nnz");
  for (int64_t r = 0; r < A.rows; r++)
    if (A.row_ptr[r + 1] < A.row_ptr[r]) return fail(SMAT_ERR_INVALID, "row_ptr not monotone");
  for (int64_t k = 0; k < A.nnz; k++)
    if (A.col_idx[k] < 0 || A.col_idx[k] >= A.cols)
      return fail(SMAT_ERR_INVALID, "column index out of range");
  if (perm) {
    std::vector<uint8_t> seen(A.rows, 0);
    for (int64_t r = 0; r < A.rows; r++) {
      if (perm[r] < 0 || perm[r] >= A.rows || seen[perm[r]])
        return fail(SMAT_ERR_INVALID, "row_perm is not a permutation");
      seen[perm[r]] = 1;
    }
  }
  out.rows = A.rows;
  out.cols = A.cols;
  out.bh = bh;
  out.bw = bw;
  out.nnz = A.nnz;
  out.rows_p = (A.rows + bh - 1) / bh * bh;
  out.cols_p = (A.cols + bw - 1) / bw * bw;
  const int64_t nbr = out.rows_p / bh, nbc = out.cols_p / bw;
  if (out.cols_p > INT32_MAX) return fail(SMAT_ERR_UNSUPPORTED, "more than 2^31 columns");

  out.row_map.assign(out.rows_p, -1);
  for (int64_t r = 0; r < A.rows; r++) out.row_map[r] = (int32_t)(perm ? perm[r] : r);

  auto src_row = [&](int64_t r) -> int64_t { return perm ? perm[r] : r; };

  // pass 1: number of nonzero blocks per block row
  std::vector<int64_t> cnt(nbr + 1, 0);
#pragma omp parallel
  {
    std::vector<int64_t> stamp(nbc, -1);
#pragma omp for schedule(dynamic, 64)
    for (int64_t br = 0; br < nbr; br++) {
      int64_t c = 0;
      for (int64_t r = br * bh; r < std::min<int64_t>((br + 1) * bh, A.rows); r++) {
        int64_t s = src_row(r);
        for (int64_t k = A.row_ptr[s]; k < A.row_ptr[s + 1]; k++) {
          int64_t bc = A.col_idx[k] / bw;
          if (stamp[bc] != br) {
            stamp[bc] = br;
            c++;
          }
        }
      }
      cnt[br + 1] = c;
    }
  }
  for (int64_t br = 0; br < nbr; br++) cnt[br + 1] += cnt[br];
  const int64_t nnzb = cnt[nbr];
  if (nnzb > INT32_MAX / 2) return fail(SMAT_ERR_UNSUPPORTED, "too many blocks");
  out.rowptr.resize(nbr + 1);
  for (int64_t br = 0; br <= nbr; br++) out.rowptr[br] = (int32_t)cnt[br];
  out.colidx.resize(nnzb);
  const int64_t bsz = (int64_t)bh * bw;
  out.val.assign(nnzb * bsz, 0.0f);
  out.val_f16.assign(nnzb * bsz, 0);
  out.is24.assign(nnzb, 0);

  // pass 2: sorted block columns, then values in CSR order
#pragma omp parallel
  {
    std::vector<int64_t> stamp(nbc, -1);
    std::vector<int32_t> slot(nbc, 0);
    std::vector<int32_t> cols;
#pragma omp for schedule(dynamic, 64)
    for (int64_t br = 0; br < nbr; br++) {
      cols.clear();
      const int64_t r1 = std::min<int64_t>((br + 1) * bh, A.rows);
      for (int64_t r = br * bh; r < r1; r++) {
        int64_t s = src_row(r);
        for (int64_t k = A.row_ptr[s]; k < A.row_ptr[s + 1]; k++) {
          int64_t bc = A.col_idx[k] / bw;
          if (stamp[bc] != br) {
            stamp[bc] = br;
            cols.push_back((int32_t)bc);
          }
        }
      }
      std::sort(cols.begin(), cols.end());
      const int64_t base = cnt[br];
      for (size_t t = 0; t < cols.size(); t++) {
        out.colidx[base + t] = cols[t] * bw;
        slot[cols[t]] = (int32_t)(base + t);
      }
      for (int64_t r = br * bh; r < r1; r++) {
        int64_t s = src_row(r);
        for (int64_t k = A.row_ptr[s]; k < A.row_ptr[s + 1]; k++) {
          int64_t col = A.col_idx[k];
          int64_t b = slot[col / bw];
          int64_t off = b * bsz + (r % bh) * bw + col % bw;
          float vf;
          uint16_t vh;
          if (!A.values) {
            vf = 1.0f;
            vh = 0x3c00;
          } else if (A.values_dtype == SMAT_F32) {
            vf = ((const float*)A.values)[k];
            vh = f32_to_f16_bits(vf);
          } else if (A.values_dtype == SMAT_F64) {
            double d = ((const double*)A.values)[k];
            vf = (float)d;
            vh = f64_to_f16_bits(d);
          } else {
            vh = ((const uint16_t*)A.values)[k];
            vf = f16_bits_to_f32(vh);
          }
          out.val[off] = vf;
          out.val_f16[off] = vh;
        }
      }
      // exact 2:4 along the block's columns, judged on the FP16 values
      for (int64_t b = base; b < cnt[br + 1]; b++) {
        const uint16_t* v = out.val_f16.data() + b * bsz;
        bool ok = (bw % 4) == 0;
        for (int rr = 0; rr < bh && ok; rr++)
          for (int g = 0; g < bw && ok; g += 4) {
            int nz = 0;
            for (int c = g; c < g + 4; c++) nz += (v[rr * bw + c] & 0x7fff) != 0;
            ok = nz <= 2;
          }
        out.is24[b] = ok ? 1 : 0;
      }
    }
  }
  return SMAT_OK;
}

smat_status build_host_bcsr_from_blocks(int64_t rows, int64_t cols, int32_t bh, int32_t bw, int64_t nnzb,
                                        const int32_t* row_ptr, const int32_t* col_idx, const uint16_t* vals,
                                        HostBcsr& out) {
  if (bh != 16 || (bw != 16 && bw != 32))
    return fail(SMAT_ERR_UNSUPPORTED, "BCSR input must have 16x16 or 16x32 blocks");
  if (rows < 0 || cols < 0 || rows % bh || cols % bw)
    return fail(SMAT_ERR_INVALID, "rows and cols must be multiples of the block shape");
  if (nnzb < 0 || !row_ptr || (nnzb > 0 && (!col_idx || !vals))) return fail(SMAT_ERR_INVALID, "BCSR arrays missing");
  const int64_t nbr = rows / bh;
  if (row_ptr[0] != 0 || row_ptr[nbr] != nnzb) return fail(SMAT_ERR_INVALID, "row_ptr[0] must be 0 and row_ptr[last] == nnzb");
  for (int64_t r = 0; r < nbr; r++) {
    if (row_ptr[r + 1] < row_ptr[r]) return fail(SMAT_ERR_INVALID, "row_ptr not monotone");
    for (int32_t k = row_ptr[r]; k < row_ptr[r + 1]; k++) {
      if (col_idx[k] < 0 || col_idx[k] >= cols || col_idx[k] % bw)
        return fail(SMAT_ERR_INVALID, "column start out of range or not a multiple of the block width");
      if (k > row_ptr[r] && col_idx[k] <= col_idx[k - 1])
        return fail(SMAT_ERR_INVALID, "block columns must ascend within a block row");
    }
  }
  if (nnzb * (bw / 16) >= ((int64_t)1 << 31) - 1) return fail(SMAT_ERR_UNSUPPORTED, "too many blocks");
  // 16-column blocks: a 16 x 32 block becomes two, both kept (a zero half
  // still multiplies B, as in the reference kernels)
  const int split = bw / 16;
  const size_t bsz = 256;
  out.rows = out.rows_p = rows;
  out.cols = out.cols_p = cols;
  out.bh = 16;
  out.bw = 16;
  out.rowptr.assign(nbr + 1, 0);
  for (int64_t r = 0; r < nbr; r++) out.rowptr[r + 1] = row_ptr[r + 1] * split;
  out.colidx.resize(nnzb * split);
  out.val.resize(nnzb * split * bsz);
  out.val_f16.resize(nnzb * split * bsz);
  out.is24.assign(nnzb * split, 0);
  int64_t nnz = 0;
#pragma omp parallel for schedule(static) reduction(+ : nnz)
  for (int64_t k = 0; k < nnzb; k++) {
    for (int h = 0; h < split; h++) {
      const int64_t b = k * split + h;
      out.colidx[b] = col_idx[k] + 16 * h;
      bool ok = true;
      for (int rr = 0; rr < 16; rr++) {
        int grp = 0;
        for (int c = 0; c < 16; c++) {
          const uint16_t v = vals[(size_t)k * 16 * bw + rr * bw + 16 * h + c];
          out.val_f16[b * bsz + rr * 16 + c] = v;
          out.val[b * bsz + rr * 16 + c] = f16_bits_to_f32(v);
          const bool nz = (v & 0x7fff) != 0;
          nnz += nz;
          grp += nz;
          if ((c & 3) == 3) {
            ok = ok && grp <= 2;
            grp = 0;
          }
        }
      }
      out.is24[b] = ok ? 1 : 0;
    }
  }
  out.nnz = nnz;
  out.row_map.resize(rows);
  for (int64_t r = 0; r < rows; r++) out.row_map[r] = (int32_t)r;
  return SMAT_OK;
}

smat_status block_info_ref(const smat_csr& A, const int64_t* perm, const HostBcsr& b, std::vector<int8_t>& info) {
  const int64_t nbr = b.nbr(), nbc = b.cols_p / b.bw;
  info.assign(b.nnzb(), 0);
#pragma omp parallel
  {
    std::vector<int32_t> where(nbc, -1);
#pragma omp for schedule(dynamic, 64)
    for (int64_t br = 0; br < nbr; br++) {
      for (int32_t k = b.rowptr[br]; k < b.rowptr[br + 1]; k++) where[b.colidx[k] / b.bw] = k;
      for (int64_t r = br * b.bh; r < std::min<int64_t>((br + 1) * b.bh, A.rows); r++) {
        const int64_t src = perm ? perm[r] : r, j0 = A.row_ptr[src], j1 = A.row_ptr[src + 1];
        for (int64_t j = j0; j < j1; j++) {
          const int64_t col = A.col_idx[j];
          int8_t& st = info[where[col / b.bw]];
          if (st == 0) {
            st = 1;  // first entry: the block starts as 2:4
          } else if (st == 1) {
            const int64_t q = col % 4;
            if ((q == 2 || q == 3) && j >= j0 + 2 && A.col_idx[j - 1] == col - 1 && A.col_idx[j - 2] == col - 2)
              st = 2;  // three consecutive columns in file order: dense
          }
        }
      }
      for (int32_t k = b.rowptr[br]; k < b.rowptr[br + 1]; k++) where[b.colidx[k] / b.bw] = -1;
    }
  }
  return SMAT_OK;
}

// Nearest e4m3 value (round to nearest even) of a in [0, 464).
static inline float e4m3_round(float a) {
  if (a < 0.015625f) return std::nearbyint(a * 512.0f) * (1.0f / 512.0f);  // subnormals: step 2^-9
  uint32_t bits;
  std::memcpy(&bits, &a, 4);
  const int e = (int)((bits >> 23) & 0xffu) - 127;                          // a in [2^e, 2^(e+1))
  const uint32_t step_bits = (uint32_t)(e - 3 + 127) << 23;                  // 2^(e-3): 3 fraction bits
  float step;
  std::memcpy(&step, &step_bits, 4);
  return std::min(448.0f, std::nearbyint(a / step) * step);
}

smat_status quantize_fp8(const HostBcsr& b, std::vector<uint8_t>& q, std::vector<float>& scale) {
  const int64_t nnzb = b.nnzb();
  const int bsz = b.bh * b.bw;
  for (float v : b.val)
    if (!(std::fabs(v) <= 65504.0f))
      return fail(SMAT_ERR_UNSUPPORTED, "FP8 form: values must be finite and within the FP16 range");
  q.assign((size_t)nnzb * bsz, 0);
  scale.assign(nnzb, 1.0f);
  // candidate maps of the block's largest magnitude: 448 down to 224 (one
  // binade), so that some scale puts the block's values on a good e4m3 grid
  constexpr int kCand = 24;
#pragma omp parallel for schedule(dynamic, 256)
  for (int64_t k = 0; k < nnzb; k++) {
    const float* v = b.val.data() + (size_t)k * bsz;
    float amax = 0.0f;
    for (int i = 0; i < bsz; i++) amax = std::max(amax, std::fabs(v[i]));
    if (amax == 0.0f) continue;
    float best_s = amax / 448.0f;
    double best_e = INFINITY;
    for (int c = 0; c < kCand; c++) {
      const float t = 448.0f - 224.0f * (float)c / (float)kCand;
      const float sc = amax / t;
      double e = 0.0;
      for (int i = 0; i < bsz; i++) {
        if (v[i] == 0.0f) continue;
        const float r = e4m3_round(std::fabs(v[i]) / sc) * sc;
        const double d = (double)r - (double)std::fabs(v[i]);
        e += d * d;
      }
      if (e < best_e) {
        best_e = e;
        best_s = sc;
      }
    }
    scale[k] = best_s;
    for (int i = 0; i < bsz; i++) q[(size_t)k * bsz + i] = v[i] == 0.0f ? 0 : f32_to_e4m3_bits(v[i] / best_s);
  }
  return SMAT_OK;
}

smat_status build_plan(const HostBcsr& b, int32_t R, int32_t cls, Plan& plan, const std::vector<uint8_t>* skip) {
  if (R < 1 || R > 32) return fail(SMAT_ERR_INVALID, "panel rows must be in [1, 32]");
  const int64_t nbr = b.nbr();
  plan.R = R;
  if (b.nnzb() >= ((int64_t)1 << 31) - 1) return fail(SMAT_ERR_UNSUPPORTED, "too many blocks");
  const int32_t SB = stage_rows(cls) / b.bh;                 // blocks per stage
  const int32_t ST = stage_tiles(cls);                       // B tiles per stage
  const int32_t max_len = std::min<int32_t>(16, kMaxGroupN / b.bh);
  // MMA-issuing warp owning a slot: kMmaWarps equal ranges of slots
  auto owner = [R](uint32_t slot) -> uint32_t { return (uint32_t)((slot * kMmaWarps) / (uint32_t)R); };

  // ---- panels and TMEM slots. A slot accumulates some blocks of one
  // block row. Each issuing warp owns a fixed range of slots; one thread
  // issues at most one MMA every ~78 cycles while the tensor pipe takes ~39
  // per narrow MMA, so a warp with more than its share of a stage's blocks
  // sets the pace. A block row holding more than a quarter of the panel's
  // blocks (a hub row) is therefore dealt over kMmaWarps parts, block k of the
  // row to part k mod kMmaWarps (every stage, a window of block columns, then
  // finds work for every warp), part w in warp w's range at the same position
  // (the epilogue adds the parts, in warp order); the other rows take the free
  // slots heaviest first, each in the warp with the fewest blocks so far. A
  // panel takes up to R consecutive block rows, fewer when its cut rows need
  // the room. A slot accumulates blocks k0, k0 + step, ... < k1.
  struct SlotSrc {
    int32_t br = -1, k0 = 0, k1 = 0, step = 1;
  };
  std::vector<SlotSrc> slots;
  std::vector<uint32_t> ext_masks;
  const int32_t per_warp = R / kMmaWarps;
  const bool can_cut = R % kMmaWarps == 0;
  auto wrow = [&b](int64_t br) { return (int64_t)(b.rowptr[br + 1] - b.rowptr[br]); };
  auto is_hub = [](int64_t w, int64_t W) { return w >= kMinCutBlocks && kMmaWarps * w > W; };
  int32_t order[32], first_free[kMmaWarps], end_free[kMmaWarps];
  int64_t load[kMmaWarps];
  for (int64_t pos = 0; pos < nbr;) {
    int32_t n = (int32_t)std::min<int64_t>(R, nbr - pos), h = 0;
    for (;; n--) {  // n = 1 always fits: a single cut row takes one position per warp
      int64_t W = 0;
      for (int32_t r = 0; r < n; r++) W += wrow(pos + r);
      h = 0;
      if (can_cut)
        for (int32_t r = 0; r < n; r++) h += is_hub(wrow(pos + r), W) ? 1 : 0;
      if (h <= per_warp && n + (kMmaWarps - 1) * h <= R) break;
    }
    int64_t W = 0;
    for (int32_t r = 0; r < n; r++) W += wrow(pos + r);
    const size_t p = ext_masks.size();
    slots.resize((p + 1) * (size_t)R);
    SlotSrc* S = &slots[p * (size_t)R];
    uint32_t ext = 0;
    for (int w = 0; w < kMmaWarps; w++) {
      load[w] = 0;
      first_free[w] = end_free[w] = -1;
    }
    for (int32_t sl = 0; sl < R; sl++) {
      const uint32_t w = owner((uint32_t)sl);
      if (first_free[w] < 0) first_free[w] = sl;
      end_free[w] = sl + 1;
    }
    int32_t nlight = 0, j = 0;
    for (int32_t r = 0; r < n; r++) {
      const int64_t br = pos + r, w_r = wrow(br);
      if (h > 0 && is_hub(w_r, W)) {
        for (int w = 0; w < kMmaWarps; w++) {
          const int32_t sl = w * per_warp + j;
          S[sl].br = (int32_t)br;
          S[sl].k0 = b.rowptr[br] + w;
          S[sl].k1 = b.rowptr[br + 1];
          S[sl].step = kMmaWarps;
          load[w] += (w_r - w + kMmaWarps - 1) / kMmaWarps;
          if (w > 0) ext |= 1u << sl;
        }
        j++;
      } else {
        order[nlight++] = r;
      }
    }
    for (int w = 0; w < kMmaWarps; w++)
      if (first_free[w] >= 0) first_free[w] += j;
    std::stable_sort(order, order + nlight, [&](int32_t x, int32_t y) { return wrow(pos + x) > wrow(pos + y); });
    for (int32_t i = 0; i < nlight; i++) {
      const int64_t br = pos + order[i];
      int best = -1;
      for (int w = 0; w < kMmaWarps; w++)
        if (first_free[w] >= 0 && first_free[w] < end_free[w] && (best < 0 || load[w] < load[best])) best = w;
      const int32_t sl = first_free[best]++;
      S[sl].br = (int32_t)br;
      S[sl].k0 = b.rowptr[br];
      S[sl].k1 = b.rowptr[br + 1];
      load[best] += wrow(br);
    }
    ext_masks.push_back(ext);
    pos += n;
  }
  plan.n_panels = (int32_t)ext_masks.size();
  const int32_t P = plan.n_panels;
  // C row of each plan row (panel * R + slot) * bh + i; parts after the first
  // of a cut row have none (the epilogue adds them into the first)
  plan.row_map.assign((size_t)P * R * b.bh, -1);
  for (size_t q = 0; q < slots.size(); q++) {
    const SlotSrc& src = slots[q];
    if (src.br < 0 || ((ext_masks[q / R] >> (q % R)) & 1u)) continue;
    for (int32_t i = 0; i < b.bh; i++) plan.row_map[q * b.bh + i] = b.row_map[(size_t)src.br * b.bh + i];
  }
  struct Local {
    std::vector<StageRec> stages;
    std::vector<uint8_t> hdr;
    std::vector<int32_t> blk;
    PanelInfo info{};
    int64_t groups = 0, tiles = 0;
  };
  std::vector<Local> loc(P);
#pragma omp parallel
  {
    std::vector<std::pair<int64_t, int32_t>> ent;  // (col * 32 + slot, block)
    std::vector<std::pair<uint32_t, uint32_t>> mma;  // (owner, entry) of the stage being built
#pragma omp for schedule(dynamic, 16)
    for (int32_t p = 0; p < P; p++) {
      Local& L = loc[p];
      ent.clear();
      const SlotSrc* S = &slots[(size_t)p * R];
      uint32_t mask = 0;
      for (int32_t sl = 0; sl < R; sl++) {
        if (S[sl].k1 > S[sl].k0) mask |= 1u << sl;
        for (int32_t k = S[sl].k0; k < S[sl].k1; k += S[sl].step)
          if (!skip || !(*skip)[k]) ent.push_back({(int64_t)b.colidx[k] * 32 + sl, k});
      }
      L.info.ext_mask = ext_masks[p];
      std::sort(ent.begin(), ent.end());
      L.info.nblk = (int32_t)ent.size();
      L.info.slot_mask = mask;
      // accumulate flags in stream order: the first block of a slot overwrites
      std::vector<uint8_t> acc(ent.size(), 0);
      uint32_t touched = 0;
      for (size_t t = 0; t < ent.size(); t++) {
        const uint32_t slot = (uint32_t)(ent[t].first % 32);
        if ((touched >> slot) & 1u) acc[t] = 1;
        touched |= 1u << slot;
      }
      // stages: whole block columns where they fit
      size_t t = 0;
      int32_t ucols = 0;
      while (t < ent.size()) {
        StageRec s{};
        mma.clear();
        while (t < ent.size() && s.ntiles < ST && s.nblk < SB) {
          const int64_t col = ent[t].first / 32;
          size_t e = t;
          while (e < ent.size() && ent[e].first / 32 == col) e++;
          const int32_t run = (int32_t)(e - t);
          const int32_t room = SB - s.nblk;
          if (run > room && s.nblk > 0 && run <= SB) break;  // keep the column whole
          const int32_t take = std::min(run, room);
          const int32_t tile = s.ntiles++;
          s.kb[tile] = (int32_t)(col / 16);
          if (t == 0 || ent[t - 1].first / 32 != col) ucols++;
          // MMA groups among the taken blocks
          for (int32_t g = 0; g < take;) {
            const uint32_t slot0 = (uint32_t)(ent[t + g].first % 32);
            int32_t len = 1;
            while (g + len < take && len < max_len) {
              const uint32_t sl = (uint32_t)(ent[t + g + len].first % 32);
              if (sl != slot0 + (uint32_t)len) break;
              if (acc[t + g + len] != acc[t + g]) break;
              if (owner(sl) != owner(slot0)) break;
              len++;
            }
            const uint32_t pos = (uint32_t)(s.nblk + g);
            const uint32_t entry = pos | ((uint32_t)tile << 5) | (slot0 << 9) | ((uint32_t)(len - 1) << 14) |
                                   (acc[t + g] ? kEntAccBit : 0u);
            mma.push_back({owner(slot0), entry});
            L.groups++;
            g += len;
          }
          for (int32_t q = 0; q < take; q++) L.blk.push_back(ent[t + q].second);
          s.nblk += take;
          t += take;
        }
        L.tiles += s.ntiles;
        // header: per-warp (first, count), nblk, then the entries grouped by warp
        std::stable_sort(mma.begin(), mma.end(),
                         [](const std::pair<uint32_t, uint32_t>& x, const std::pair<uint32_t, uint32_t>& y) {
                           return x.first < y.first;
                         });
        const int32_t ne = (int32_t)mma.size();
        s.hdr_bytes = (kStageHdrFixed + 4 * ne + 15) / 16 * 16;
        const size_t h0 = L.hdr.size();
        L.hdr.resize(h0 + s.hdr_bytes, 0);
        uint8_t* h = L.hdr.data() + h0;
        uint16_t wl[kMmaWarps] = {0, 0, 0, 0};
        for (int32_t i = 0; i < ne; i++) {
          const uint32_t w = mma[i].first;
          if ((wl[w] >> 8) == 0) wl[w] = (uint16_t)i;
          wl[w] = (uint16_t)((wl[w] & 0xffu) | (((wl[w] >> 8) + 1u) << 8));
          std::memcpy(h + kStageHdrFixed + 4 * i, &mma[i].second, 4);
        }
        std::memcpy(h, wl, sizeof(wl));
        const uint16_t nb16 = (uint16_t)s.nblk, nt16 = (uint16_t)s.ntiles;
        std::memcpy(h + 8, &nb16, 2);
        std::memcpy(h + 10, &nt16, 2);
        L.stages.push_back(s);
      }
      L.info.nstages = (int32_t)L.stages.size();
      L.info.nucol = ucols;
    }
  }
  // concatenate
  int64_t nst = 0, nb = 0, nh = 0;
  for (auto& L : loc) {
    nst += (int64_t)L.stages.size();
    nb += (int64_t)L.blk.size();
    nh += (int64_t)L.hdr.size();
  }
  if (nst >= ((int64_t)1 << 31) || (int64_t)nb * 4 + nst * 16 >= ((int64_t)1 << 31))
    return fail(SMAT_ERR_UNSUPPORTED, "plan too large");
  plan.panels.resize(P);
  plan.stages.resize(nst);
  plan.stream_blk.resize(nb);
  plan.headers.resize(nh);
  plan.n_groups = 0;
  plan.n_tiles = 0;
  int64_t so = 0, bo = 0, ho = 0, xo = 0;
  for (int32_t p = 0; p < P; p++) {
    Local& L = loc[p];
    L.info.stage_off = (int32_t)so;
    plan.panels[p] = L.info;
    std::copy(L.blk.begin(), L.blk.end(), plan.stream_blk.begin() + bo);
    std::copy(L.hdr.begin(), L.hdr.end(), plan.headers.begin() + ho);
    for (size_t c = 0; c < L.stages.size(); c++) {
      StageRec r = L.stages[c];
      r.blk_off = bo;
      r.hdr_off = ho;
      r.scl_off = (int32_t)xo;
      bo += r.nblk;
      ho += r.hdr_bytes;
      xo += fp8_scale_bytes(r.nblk);
      plan.stages[so + c] = r;
    }
    so += (int64_t)L.stages.size();
    plan.n_groups += L.groups;
    plan.n_tiles += L.tiles;
  }
  return SMAT_OK;
}

void build_work_items_multi(const std::vector<const Plan*>& plans, const std::vector<int32_t>& bhs, int32_t workers,
                            double max_item_frac, std::vector<WorkItem>& items, std::vector<int32_t>& order,
                            std::vector<int32_t>& n_split, std::vector<int32_t>& n_slabs) {
  // cost of a stage in units of one A block: the block copies, the B tiles
  // (a 4 KB tile moves 8x the bytes of a block, from L2) and a fixed
  // per-stage hand-off cost; per item, the epilogue (R * bh rows of C)
  auto stage_cost = [](const StageRec& r) { return r.nblk + 2.0 * r.ntiles + 4.0; };
  const int32_t np = (int32_t)plans.size();
  std::vector<std::vector<double>> pcost(np);
  double total = 0.0;
  for (int32_t q = 0; q < np; q++) {
    const Plan& pl = *plans[q];
    pcost[q].assign(pl.n_panels, 0.0);
    for (int32_t p = 0; p < pl.n_panels; p++) {
      for (int32_t c = 0; c < pl.panels[p].nstages; c++)
        pcost[q][p] += stage_cost(pl.stages[pl.panels[p].stage_off + c]);
      pcost[q][p] += 0.5 * pl.R * bhs[q];
      total += pcost[q][p];
    }
  }
  double max_item = std::max(1.0, max_item_frac * total / std::max(1, workers));
  // a part costs a full epilogue, a slab write and a share of the fixup
  // whatever its size: never cut a panel into parts of fewer than
  // kMinPartStages stages (small matrices then keep whole panels)
  constexpr int32_t kMinPartStages = 4;
  auto max_parts = [](int32_t nstages) { return std::max<int32_t>(1, nstages / kMinPartStages); };
  // bound the partial-sum slabs: at most kMaxSlabs parts of split panels per
  // problem (coarser parts where a problem would need more)
  constexpr int64_t kMaxSlabs = 96;
  for (int32_t q = 0; q < np; q++) {
    for (int iter = 0; iter < 64; iter++) {
      int64_t parts_q = 0;
      for (int32_t p = 0; p < plans[q]->n_panels; p++) {
        const int64_t parts = std::min<int64_t>((int64_t)std::ceil(pcost[q][p] / max_item),
                                                max_parts(plans[q]->panels[p].nstages));
        if (parts > 1) parts_q += parts;
      }
      if (parts_q <= kMaxSlabs) break;
      max_item *= 1.25;
    }
  }
  items.clear();
  n_split.assign(np, 0);
  n_slabs.assign(np, 0);
  std::vector<double> icost;
  for (int32_t q = 0; q < np; q++) {
    const Plan& pl = *plans[q];
    const double epi = 0.5 * pl.R * bhs[q];
    for (int32_t p = 0; p < pl.n_panels; p++) {
      const PanelInfo& pi = pl.panels[p];
      int32_t parts = (int32_t)std::ceil(pcost[q][p] / max_item);
      parts = std::max(1, std::min(parts, max_parts(pi.nstages)));
      if (parts == 1) {
        items.push_back(WorkItem{p, 0, pi.nstages, -1, 0, 1, 0, q});
        icost.push_back(pcost[q][p]);
        continue;
      }
      // cut the stages into `parts` ranges of about equal cost
      const double per = (pcost[q][p] - epi) / parts;
      int32_t s0 = 0, part = 0;
      double acc = 0.0;
      for (int32_t c = 0; c < pi.nstages; c++) {
        acc += stage_cost(pl.stages[pi.stage_off + c]);
        const bool cut = acc >= per * (part + 1) && part < parts - 1 && c + 1 < pi.nstages;
        if (cut || c + 1 == pi.nstages) {
          items.push_back(WorkItem{p, s0, c + 1, n_split[q], part, 0, n_slabs[q], q});
          part++;
          s0 = c + 1;
        }
      }
      for (int32_t i = (int32_t)items.size() - part; i < (int32_t)items.size(); i++) {
        items[i].nparts = part;
        double c = 0.0;
        for (int32_t st = items[i].s0; st < items[i].s1; st++) c += stage_cost(pl.stages[pi.stage_off + st]);
        icost.push_back(c + 2.0 * epi);  // a part writes its slab; the last one also reads all parts back
      }
      n_split[q]++;
      n_slabs[q] += part;
    }
  }
  order_items(icost, order);
}

void build_work_items(const Plan& pl, int32_t bh, int32_t workers, double max_item_frac,
                      std::vector<WorkItem>& items, std::vector<int32_t>& order, int32_t& n_split,
                      int32_t& n_slabs) {
  std::vector<int32_t> ns, nl;
  build_work_items_multi({&pl}, {bh}, workers, max_item_frac, items, order, ns, nl);
  n_split = ns[0];
  n_slabs = nl[0];
}

void order_items(const std::vector<double>& cost, std::vector<int32_t>& order) {
  order.resize(cost.size());
  std::iota(order.begin(), order.end(), 0);
  std::stable_sort(order.begin(), order.end(), [&](int32_t a, int32_t b) { return cost[a] > cost[b]; });
}

}  // namespace smat
