/*
 * smat.h — C ABI of libsmat, a GB300 (sm_103a) implementation of the SMaT
 * pipeline: Jaccard row reordering -> BCSR blocking -> block-sparse x dense
 * SpMM on tcgen05 tensor cores.
 *
 * Conventions
 *  - Every entry point returns an smat_status; smat_last_error() gives a
 *    one-line message for the calling thread's last failure. Nothing here
 *    calls exit().
 *  - Host pointers are marked (host), device pointers (device).
 *  - Device work is enqueued on the given stream (a cudaStream_t passed as
 *    void*; NULL = legacy default stream) and is asynchronous.
 *  - smat_spmm allocates nothing and synchronises nothing; scratch for the
 *    forms that convert B is passed in by the caller.
 *
 * Each entry point names the reference interface it replaces
 * (paths inside ajit283/sptc-smat).
 */
#ifndef SMAT_H_
#define SMAT_H_

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum smat_status {
  SMAT_OK = 0,
  SMAT_ERR_INVALID = 1,     /* malformed argument or matrix */
  SMAT_ERR_UNSUPPORTED = 2, /* option or shape not implemented */
  SMAT_ERR_CUDA = 3,        /* CUDA runtime / driver error */
  SMAT_ERR_NOMEM = 4,       /* host or device allocation failed */
  SMAT_ERR_TIMEOUT = 5,     /* a bounded device-side wait expired */
  SMAT_ERR_NO_DEVICE = 6    /* no usable sm_103 device / kernels not loadable */
} smat_status;

typedef enum smat_dtype {
  SMAT_F32 = 0,
  SMAT_F16 = 1,
  SMAT_BF16 = 2,
  SMAT_F64 = 3,
  SMAT_E4M3 = 4
} smat_dtype;

/* Arithmetic form of the SpMM. All forms accumulate in FP32 (TMEM). */
typedef enum smat_form {
  SMAT_FORM_F16 = 0,        /* FP16 A and B (the plain form) */
  SMAT_FORM_BF16 = 1,       /* BF16 A and B */
  SMAT_FORM_FP8 = 2,        /* e4m3 A with one FP32 scale per block */
  SMAT_FORM_SPLIT_BF16 = 3  /* hi+lo BF16 A and B, three products */
} smat_form;

typedef enum smat_layout { SMAT_ROW_MAJOR = 0, SMAT_COL_MAJOR = 1 } smat_layout;

/* A sparse matrix in CSR (host). Column indices within a row are kept in the
 * given order ("file order"); values may be NULL (pattern: every value 1). */
typedef struct smat_csr {
  int64_t rows;
  int64_t cols;
  int64_t nnz;
  const int64_t* row_ptr; /* (host) rows + 1 */
  const int32_t* col_idx; /* (host) nnz */
  const void* values;     /* (host) nnz elements of values_dtype, or NULL */
  int32_t values_dtype;   /* SMAT_F32, SMAT_F16 or SMAT_F64 */
} smat_csr;

/* BCSR build options. */
typedef struct smat_bcsr_opts {
  int32_t block_rows;     /* bh: 16 (default when 0) */
  int32_t block_cols;     /* bw: 16 (default when 0) */
  uint32_t forms;         /* bit (1 << smat_form) per form to materialise; 0 = F16 only */
  int32_t use_24;         /* 0: off. k > 0: a block that is exactly 2:4 (at most two nonzeros
                             in every aligned group of four columns of every row) runs on the
                             structured-sparse tensor-core path (FP16 / BF16 forms, 16 x 16
                             blocks) when its unit -- 8 block rows x one 32-column window --
                             holds at least k such blocks; 1 = every such block, as the
                             reference routes them (mmaOBTS_large.cu:19-254); the other
                             blocks stay on the dense path */
  const int64_t* row_perm;/* (host, optional) new row r = old row row_perm[r]; SpMM results
                             are written back in the ORIGINAL row order */
  int32_t device;         /* CUDA device ordinal */
  int32_t panel_rows;     /* block rows per tensor-core panel: 4, 8 or 16 for bh 16, 4 or 8
                             for bh 32; 0 = the autotuner's cached choice for matrices
                             like this one, else 256 rows (16, or 8 for bh 32) */
  float split_frac;       /* a panel costing more than split_frac x the average per-CTA
                             work is split into parts over several CTAs (0 = default 0.5,
                             < 0 = never split) */
  const int64_t* col_perm;/* (host, optional) new column c = old column col_perm[c]: A is
                             blocked with its columns permuted (the reference's column
                             reordering, src/reorder.py:140-182) and smat_spmm gathers B's
                             rows through the same permutation, so C = A * B unchanged;
                             smat_bcsr_export then shows the permuted columns */
  int32_t n_tile_cols;    /* 0 or 128: C is computed 128 columns per pass over A; 256: with
                             panel_rows <= 8 the handle also holds a plan for 256-column
                             passes, which the FP16 and BF16 forms use for N > 128 (A read
                             once per 256 columns; one more copy of A on the device);
                             with panel_rows = 0 the autotuner's cached choice */
  int32_t pipeline_depth; /* pipeline stages in flight (2..): 0 = as many as fit in shared
                             memory (3 for the default stage shapes), or the autotuner's
                             cached choice when panel_rows = 0 */
} smat_bcsr_opts;

typedef struct smat_bcsr smat_bcsr; /* opaque handle, immutable after create */

typedef struct smat_bcsr_info {
  int64_t rows, cols;           /* logical (unpadded) shape */
  int64_t rows_padded, cols_padded;
  int64_t nnz;                  /* scalar nonzeros stored in the input CSR */
  int64_t nnzb;                 /* nonzero blocks */
  int64_t n_blocks_24;          /* blocks routed to the 2:4 path (0 unless use_24) */
  int32_t block_rows, block_cols;
  int32_t panel_rows;
  int32_t n_panels;
  int64_t n_union_cols;         /* B tiles one SpMM pass loads (per N tile) */
  double fill;                  /* nnz / (nnzb * bh * bw) */
  int32_t n_tile_cols;          /* widest N tile the handle runs: 128, or 256 (FP16 / BF16, N > 128) */
  int32_t pipeline_depth;       /* stages in flight requested (0: all that fit) */
} smat_bcsr_info;

typedef struct smat_reorder_stats {
  int64_t comparisons;          /* distance evaluations (blocking.cpp comparison_counter) */
  int64_t merges;               /* rows merged under tau (merge_counter) */
} smat_reorder_stats;

/* ---------------------------------------------------------------- files */

/* A CSR read from a file; the arrays belong to the library (release them
 * with smat_csr_file_free). */
typedef struct smat_csr_file {
  smat_csr csr;       /* values: SMAT_F64 from MatrixMarket, SMAT_F32 from edge lists, NULL for patterns */
  int32_t symmetric;  /* MatrixMarket symmetric/hermitian file, expanded */
} smat_csr_file;

/* MatrixMarket coordinate file -> CSR, as mmio_allinone + padSparseMatrix
 * (src/cuda_hgemm/src/common/mmio_highlevel.h:514-680): rows padded to a
 * multiple of 16, columns to a multiple of col_pad (the block width), entries
 * in file order, symmetric/hermitian files mirrored (the mirrored entry right
 * after its source), complex files keep the real part, pattern values 1.0.
 * Values are the parsed doubles (FP16 conversion happens once, later). */
smat_status smat_read_mtx(const char* path, int32_t col_pad, smat_csr_file* out);

/* Edge list "row col [value]" -> CSR, as CSR::read_from_edgelist
 * (preprocess/src/general/csr.cpp:166-290) with its defaults (space
 * delimiter, general matrix): rows ascending, cols = max column + 1, FP32
 * values unless pattern_only. */
smat_status smat_read_el(const char* path, int32_t pattern_only, smat_csr_file* out);

/* Pattern edge list of A with new row r = old row row_perm[r] (NULL: as is):
 * the *_reordered.el file Matrix_Blocking writes (csr.cpp:150-161). */
smat_status smat_write_el(const char* path, const smat_csr* A, const int64_t* row_perm);

smat_status smat_csr_file_free(smat_csr_file* f);

/* ---------------------------------------------------------------- step 1 */

/* Row reordering. Replaces `Matrix_Blocking -f x.el -a algo -b col_block
 * -B row_block -F force_fixed -t tau` (preprocess/test/general/Matrix_Blocking.cpp:10-50,
 * driven by src/reorder.py:131-132) and in-process
 * BlockingEngine::GetGrouping + CSR::reorder (preprocess/src/general/blocking.cpp:616-657,
 * csr.cpp:97-105). algo 5 (IterativeBlockingKeeper, the pipeline's choice)
 * and 2 (fixed size) are supported. perm_out[r] = old row placed at new row r,
 * identical to the reference's permutation; grouping_out (optional) receives
 * the final grouping vector (the reference's ".g" file content). A column
 * index is "the" column (col_idx); the pattern is used, values are ignored.
 * use_gpu = 0: the candidate distances of the scan run on the host's cores;
 * use_gpu != 0: on the current CUDA device, in larger chunks (the seed loop
 * and its commits stay on the host), with the same result. */
smat_status smat_reorder(const smat_csr* A, float tau, int32_t col_block, int32_t row_block,
                         int32_t algo, int32_t force_fixed, int32_t use_gpu, int64_t* perm_out,
                         int64_t* grouping_out, smat_reorder_stats* stats);

/* ---------------------------------------------------------------- step 2 */

/* CSR -> BCSR, uploaded to the device. Replaces the SparseMatrix constructor
 * (src/cuda_hgemm/src/common/matrix.h:161-246: csrToBcsr :666-792 and
 * filterBcsrBlocks :1140-1288). Rows are padded to a multiple of bh and
 * columns to a multiple of bw (mmio_highlevel.h:514-520). The block structure
 * and values are bit-identical to csrToBcsr on the (optionally permuted) CSR. */
smat_status smat_bcsr_create(const smat_csr* A, const smat_bcsr_opts* opts, smat_bcsr** out);
/* The same handle from an existing BCSR on the host: the arrays the
 * reference's SparseMatrix keeps (getBcsrRowPtrHost / getBcsrColIdxHost /
 * getBcsrValuesHost, matrix.h:475-477): row_ptr[rows/16 + 1], col_idx[nnzb]
 * (column starts, ascending in each block row), values_f16[nnzb*16*bw] (FP16
 * bits, row-major per block). Blocks are 16 x 16 or 16 x 32 (block_cols 32,
 * the reference's "large" blocks, split into two 16 x 16 blocks); rows and
 * cols are multiples of the block shape. opts.row_perm must be NULL. */
smat_status smat_bcsr_create_from_bcsr(int64_t rows, int64_t cols, int32_t block_rows, int32_t block_cols,
                                       int64_t nnzb, const int32_t* row_ptr, const int32_t* col_idx,
                                       const uint16_t* values_f16, const smat_bcsr_opts* opts, smat_bcsr** out);
smat_status smat_bcsr_destroy(smat_bcsr* A);
smat_status smat_bcsr_get_info(const smat_bcsr* A, smat_bcsr_info* info);

/* Copy the block structure back to the host (for checking against the
 * reference): row_ptr[rows_padded/bh + 1], col_idx[nnzb] (column START of
 * each block, as bcsrColIdx in matrix.h:743), values[nnzb*bh*bw] as FP16 bit
 * patterns, row-major inside each block. Any pointer may be NULL. */
smat_status smat_bcsr_export(const smat_bcsr* A, int32_t* row_ptr, int32_t* col_idx,
                             uint16_t* values_f16, uint8_t* is_24);

/* The FP8 form's data, BCSR block order: codes[nnzb*256] e4m3 (OCP "e4m3fn")
 * codes of value / scale, row-major per block, and scales[nnzb]; the SpMM
 * uses FP16(code value * scale). Each block's scale is chosen on the host to
 * minimise the block's squared quantisation error. */
smat_status smat_bcsr_export_fp8(const smat_bcsr* A, uint8_t* codes, float* scales);

/* Host-only CSR -> BCSR (no device needed): the block structure that
 * smat_bcsr_create uploads, bit-identical to SparseMatrix::csrToBcsr
 * (matrix.h:666-792) on the (optionally permuted) CSR. Call once with
 * row_ptr == NULL to get *nnzb, then again with row_ptr[rows_padded/bh + 1],
 * col_idx[nnzb] and values_f16[nnzb*bh*bw]. */
smat_status smat_csr_to_bcsr_host(const smat_csr* A, int32_t block_rows, int32_t block_cols,
                                  const int64_t* row_perm, int64_t* nnzb, int32_t* row_ptr,
                                  int32_t* col_idx, uint16_t* values_f16);

/* The reference's 2:4 / dense split of the blocks (filterBcsrBlocks,
 * matrix.h:1140-1288, with the blockInfo labels of csrToBcsr :679-711),
 * host only, bit-identical: blocks the reference labels 1 ("2:4": no row of
 * the block holds three consecutive columns in file order ending at a
 * column % 4 of 2 or 3) go to the first BCSR, the others (2, dense) to the
 * second, each in block-row and column order; block_info (optional) gets
 * the label grid [rows_padded/16][cols_padded/block_cols] (0 = empty).
 * 16-row blocks, block_cols 16 or 32. Call with row_ptr_24 == NULL for the
 * counts. */
smat_status smat_csr_to_bcsr_split_host(const smat_csr* A, int32_t block_cols, const int64_t* row_perm,
                                        int64_t* n_24, int64_t* n_dense, int32_t* row_ptr_24, int32_t* col_idx_24,
                                        uint16_t* values_24, int32_t* row_ptr_dense, int32_t* col_idx_dense,
                                        uint16_t* values_dense, int32_t* block_info);

/* The reference's merged 4 x 4-block tiles (SparseMatrix::bcsrBlocking,
 * src/cuda_hgemm/src/common/matrix.h:794-1137, whose output feeds the
 * `_tiled` launchers mmaOBTKernel_tiled / mmaOBTSKernel_tiled_large), built
 * on the GPU from a DEVICE BCSR as csrToBcsr lays it out: row_ptr[rows/16+1],
 * col_idx[nnzb] (column starts, ascending in each block row),
 * values[nnzb*16*block_cols] FP16 bits row-major per block (16-byte
 * aligned); block_cols 16 or 32; rows a multiple of 16, cols of block_cols.
 * The result is bit-identical to the reference's merged arrays:
 *   values     [n_tiles][4][4][16][block_cols] FP16 bits (block-major tiles,
 *              tiles numbered in order of first appearance in BCSR order)
 *   row_ptr    [n_rowptr]: one entry per tile row holding a tile, then
 *              n_tiles (tile rows without a tile get no entry, as there)
 *   col_idx    [n_tiles]: column start of each tile (a multiple of 4k)
 *   block_info [tile_rows * tile_cols]: 1 where a tile exists
 *   rel_map    [tile_rows * tile_cols]: tile rank in grid order, or -1
 *   tile_info  [n_tiles * 16]: the reference's 0 / 1 / 2 labels, computed as
 *              it computes them (the tile read as a row-major 64 x 4k matrix)
 * with tile_rows = ceil(rows/64), tile_cols = ceil(cols/(4*block_cols)).
 * The three input arrays are device (or managed) memory of the current
 * device. Runs on `stream` and synchronises it (the tile count sizes the
 * outputs); allocates its outputs and scratch on the current device.
 * Invalid row pointers or column starts give SMAT_ERR_INVALID. */
typedef struct smat_tiles smat_tiles; /* opaque, owns the device arrays */
typedef struct smat_tiles_desc {
  int64_t rows, cols;
  int32_t block_cols;
  int32_t device;
  int64_t n_tiles, n_rowptr, tile_rows, tile_cols;
  const uint16_t* values;     /* (device) */
  const int32_t* row_ptr;     /* (device) */
  const int32_t* col_idx;     /* (device) */
  const int32_t* block_info;  /* (device) */
  const int32_t* rel_map;     /* (device) */
  const int32_t* tile_info;   /* (device) */
} smat_tiles_desc;
smat_status smat_tiles_create(int64_t rows, int64_t cols, int32_t block_cols, int64_t nnzb,
                              const int32_t* row_ptr, const int32_t* col_idx, const void* values,
                              void* stream, smat_tiles** out);
smat_status smat_tiles_describe(const smat_tiles* t, smat_tiles_desc* out);
/* Host copies of the arrays above (any pointer may be NULL), sized as
 * described: the reference's mergedBcsr*_host / merged*_host arrays. */
smat_status smat_tiles_copy_to_host(const smat_tiles* t, int32_t* row_ptr, int32_t* col_idx, uint16_t* values,
                                    int32_t* block_info, int32_t* rel_map, int32_t* tile_info);
smat_status smat_tiles_destroy(smat_tiles* t);

/* ---------------------------------------------------------------- step 3 */

/* Bytes of device scratch smat_spmm needs for this form / B dtype / N: the
 * packed copy of B (twice that for the split form), and for panels split
 * over several CTAs for load balance, one counter per split panel and a
 * partial-sum slab per part. */
smat_status smat_spmm_workspace_size(const smat_bcsr* A, int32_t form, int32_t b_dtype, int64_t N,
                                     size_t* bytes);

/* C = A * B on the tensor cores. Replaces the launchers with the
 * HGEMM_FUNC_SPARSE2 / HGEMM_FUNC_SPARSE24_2 signatures
 * (src/cuda_hgemm/src/main.cu:20-28; mmaOBT.cu:160-169, mmaOBTS_large.cu:256-266).
 *  B (device): K x N, K = A's column count; element (k, n) at
 *     B[k + n*ldb] (SMAT_COL_MAJOR, the reference layout) or
 *     B[k*ldb + n] (SMAT_ROW_MAJOR). b_dtype: F16 for SMAT_FORM_F16, BF16 for
 *     SMAT_FORM_BF16, or F32 for any form; it is packed into workspace first.
 *  C (device): rows x N, row-major, C[i*ldc + n], c_dtype F32 or F16; rows
 *     in the ORIGINAL order when the handle was built with row_perm.
 *  workspace (device): smat_spmm_workspace_size() bytes, 256-byte aligned. */
smat_status smat_spmm(const smat_bcsr* A, int32_t form, const void* B, int32_t b_dtype,
                      int32_t b_layout, int64_t ldb, void* C, int32_t c_dtype, int64_t ldc,
                      int64_t N, void* workspace, size_t workspace_bytes, void* stream);

/* The two halves of smat_spmm, for callers that reuse one B with several
 * matrices or want to time the contraction alone: smat_spmm_pack_b writes B
 * into `workspace` in the tensor-core tile layout (4 KB tiles of 16 rows x
 * 128 columns, 32-byte swizzled, ordered [column tile][k-block] so that the
 * tiles of consecutive k-blocks are contiguous; 8 KB hi+lo pairs for the
 * split form);
 * smat_spmm_packed runs the contraction from that packed copy. */
smat_status smat_spmm_pack_b(const smat_bcsr* A, int32_t form, const void* B, int32_t b_dtype,
                             int32_t b_layout, int64_t ldb, int64_t N, void* workspace,
                             size_t workspace_bytes, void* stream);
smat_status smat_spmm_packed(const smat_bcsr* A, int32_t form, const void* packed_b, int64_t N,
                             void* C, int32_t c_dtype, int64_t ldc, void* stream);

/* Largest scratch smat_spmm_static_scratch can use (per device). */
#define SMAT_SPMM_STATIC_SCRATCH_BYTES (32u << 20)

/* smat_spmm for callers that can neither allocate device memory nor pass
 * scratch in: a launcher bound to a fixed signature without a workspace
 * parameter, or code where allocating is not allowed (cudaMalloc may
 * synchronise the device; some services fix their memory at start-up).
 * No counterpart in the reference (its launchers allocate nothing because
 * they need no scratch). Same arguments and results as smat_spmm, without
 * workspace; the packed B goes to a fixed device array of
 * SMAT_SPMM_STATIC_SCRATCH_BYTES inside the library, and nothing is
 * allocated. Returns SMAT_ERR_UNSUPPORTED when smat_spmm_workspace_size()
 * exceeds that size (the packed B, K x N x 2 bytes or twice that for the
 * split form, plus the partial sums of panels split for load balance). The
 * first call on a device looks the array's address
 * up (make it before any stream capture), and so does the first call after
 * the device's context was destroyed and created again (cudaDeviceReset).
 * All calls on a device share the
 * array: calls that overlap in time (other streams, other threads) race. */
smat_status smat_spmm_static_scratch(const smat_bcsr* A, int32_t form, const void* B, int32_t b_dtype,
                                     int32_t b_layout, int64_t ldb, void* C, int32_t c_dtype, int64_t ldc,
                                     int64_t N, void* stream);

/* ---------------------------------------------------------------- autotuner */

typedef struct smat_tune_result {
  int32_t panel_rows;   /* block rows per panel (block rows per CTA work item) that measured fastest */
  float split_frac;     /* panel splitting threshold that measured fastest (< 0: none) */
  double ms;            /* its SpMM time (pack B + contraction), milliseconds */
  double ms_default;    /* the default shape's time, for comparison (0 if cached) */
  int32_t cached;       /* 1: answered from the cache without measuring */
  int32_t n_tile_cols;  /* N-tile width that measured fastest: 128 or 256 */
  int32_t pipeline_depth; /* stages in flight that measured fastest (0: all that fit) */
  int32_t candidates;   /* shapes measured (0 if cached) */
} smat_tune_result;

/* Measures the launch shapes offered for A on opts->device for this form and
 * N -- block rows per panel x panel-splitting threshold x N-tile width (128,
 * or 256 when N > 128 and the panel has at most 8 block rows), then the
 * pipeline depth of the best of those -- and keeps the fastest in a
 * process-wide cache keyed on A's block-density statistics (blocks per
 * block row, blocks per B tile in a 16-row panel), the N-tile count and the
 * form's kernel. Later smat_bcsr_create calls with panel_rows = 0 use the
 * cached shape for matrices with the same statistics. No counterpart in the
 * reference (its tile shape is fixed at compile time). Allocates device
 * memory for its trial runs and synchronises. */
smat_status smat_autotune(const smat_csr* A, const smat_bcsr_opts* opts, int32_t form, int64_t N,
                          smat_tune_result* out);
smat_status smat_autotune_clear(void);

/* 64 values describing A for the tau / block-shape predictor, computed on
 * `device`: a row-length histogram, a bandwidth profile, the fill histogram
 * of the nonzero 16 x 16 tiles and scalar statistics (layout in
 * sptc-smat_gb300/csrc/features.cu). No counterpart in the reference. */
smat_status smat_features(const smat_csr* A, int32_t device, float* out64);

/* ------------------------------------------------- learned tau / block choice */

/* A 64-128-128-12 FP32 MLP (ReLU hidden layers) predicting, from
 * smat_features, the reordering threshold tau in {0.1, ..., 0.9} (logits
 * 0..8) and the block shape {8x8, 16x16, 32x16} (logits 9..11); trained with
 * the sum of the two heads' softmax cross-entropies and Adam, forward,
 * backward and update all in libsmat's own kernels. Inputs and outputs are
 * host arrays. No counterpart in the reference. */
typedef struct smat_mlp smat_mlp;
smat_status smat_mlp_create(int32_t device, uint64_t seed, smat_mlp** out);
int32_t smat_mlp_num_params(void);
smat_status smat_mlp_get_params(const smat_mlp* m, float* params);
smat_status smat_mlp_set_params(smat_mlp* m, const float* params);
/* Loss and gradient (parameter layout as the parameters) of one batch. */
smat_status smat_mlp_gradients(smat_mlp* m, const float* X, const int32_t* y_tau, const int32_t* y_block,
                               int32_t batch, float* grads, float* loss);
/* One Adam step (lr, beta 0.9 / 0.999, eps 1e-8) on one batch. */
smat_status smat_mlp_train_step(smat_mlp* m, const float* X, const int32_t* y_tau, const int32_t* y_block,
                                int32_t batch, float lr, float* loss);
smat_status smat_mlp_predict(smat_mlp* m, const float* X, int32_t batch, float* logits);
smat_status smat_mlp_destroy(smat_mlp* m);

/* ---------------------------------------------------------------- groups */

/* One SpMM of a group: C = A * B with the arguments of smat_spmm. */
typedef struct smat_problem {
  const smat_bcsr* A;
  int32_t form;
  const void* B;      /* (device) */
  int32_t b_dtype;
  int32_t b_layout;
  int64_t ldb;
  void* C;            /* (device) */
  int32_t c_dtype;
  int64_t ldc;
  int64_t N;
} smat_problem;

typedef struct smat_group smat_group;

/* Many SpMMs of uneven sizes in one persistent launch (no counterpart in the
 * reference, which runs one matrix at a time). smat_group_create builds, once,
 * one load-balanced work list over all the problems' block-row panels, their
 * descriptors and scratch (device memory owned by the group); B and C
 * pointers are fixed here. All handles must be on one device. */
smat_status smat_group_create(const smat_problem* problems, int32_t count, smat_group** out);
/* Runs the group on `stream`: one grouped B-packing launch, one counter
 * clear, one SpMM launch per kernel variant among the problems (one for
 * FP16/BF16 problems with N <= 128). Allocates and synchronises nothing, so
 * it can be captured in a CUDA graph (after a first run outside capture). */
smat_status smat_group_run(smat_group* g, void* stream);
/* As smat_bcsr_check_device_error, for the group's launches. */
smat_status smat_group_check_device_error(smat_group* g);
smat_status smat_group_destroy(smat_group* g);

/* Host-buffer variant: B and C in host memory; returns when C is written.
 * When both are page-locked (cudaHostAlloc / cudaMallocHost / registered),
 * the kernels read B and write C in place over the CPU-GPU link (GB300:
 * NVLink-C2C); otherwise B is copied in and C out through device buffers
 * cached in the handle. */
smat_status smat_spmm_host(const smat_bcsr* A, int32_t form, const void* B_host, int32_t b_dtype,
                           int32_t b_layout, int64_t ldb, void* C_host, int32_t c_dtype,
                           int64_t ldc, int64_t N, void* stream);

/* Reads and clears the handle's device-side error word, which the kernels
 * set when a bounded wait expires (then SMAT_ERR_TIMEOUT is returned, and
 * smat_last_error() names the wait's site). Call after synchronising the
 * stream the SpMM ran on. */
smat_status smat_bcsr_check_device_error(const smat_bcsr* A);

/* Limit, in nanoseconds, of every device-side wait in this handle's SpMM
 * launches (0: the default, 4 s). A wait that runs out aborts the launch:
 * the kernel drains its own copies and MMAs, frees its tensor memory and
 * returns, and smat_bcsr_check_device_error reports SMAT_ERR_TIMEOUT; the
 * handle stays usable. No counterpart in the reference, whose waits are
 * unbounded. */
smat_status smat_bcsr_set_wait_limit(smat_bcsr* A, uint64_t ns);

/* Testing hook for the path above: the next SpMM launch on A makes the
 * first MMA-issuing thread of CTA 0 wait, before its stage-th stage
 * (1-based), on a barrier that nothing arrives at, so that its bounded
 * wait runs out (site 205) without any fault. 0 cancels. No counterpart in
 * the reference. */
smat_status smat_bcsr_debug_stall(smat_bcsr* A, int32_t stage);

const char* smat_last_error(void);
const char* smat_version(void);

#ifdef __cplusplus
}
#endif
#endif /* SMAT_H_ */
