"""The reference's kernel launchers exported by libsmat (include/smat_ref_shims.h).

CPU: every launcher main.cu declares for the SMaT path is exported with the
reference's exact C++ signature (src/cuda_hgemm/src/main.cu:10-75).
GPU: each launcher, called the way tester.h calls it (device BCSR arrays of
the reference layout, B column-major FP16, C row-major FP16), against the
FP64 product (1e-3 relative Frobenius, FP16 output) and against the
reference's own kernel / compressor run from oracle/_ref on the same inputs
(the compressor bit for bit).
"""
import subprocess

import numpy as np
import pytest

torch = pytest.importorskip("torch")

# demangled exactly as the reference declares them
EXPECTED = {
    "mmaOBTKernel(__half*, int*, int*, __half*, __half*, unsigned long, unsigned long, unsigned long, "
    "unsigned long, int*, int*)",
    "mmaOBTKernel_large(__half*, int*, int*, __half*, __half*, unsigned long, unsigned long, unsigned long, "
    "unsigned long, int*, int*)",
    "mmaOBTSKernel(__half*, int*, int*, char*, __half*, __half*, __half*, unsigned long, unsigned long, "
    "unsigned long, unsigned long, int*, int*)",
    "mmaOBTSKernel_large(__half*, int*, int*, char*, __half*, __half*, __half*, unsigned long, unsigned long, "
    "unsigned long, unsigned long, int*, int*)",
    "mmaOBTSKernel_large_separate(__half*, int*, int*, __half*, int*, int*, char*, __half*, __half*, __half*, "
    "unsigned long, unsigned long, unsigned long, unsigned long, int*, int*)",
    "mmaOBTKernel_tiled(__half*, int*, int*, __half*, __half*, unsigned long, unsigned long, unsigned long, "
    "unsigned long, int*, int*)",
    "mmaOBTSKernel_tiled_large(__half*, int*, int*, char*, __half*, __half*, __half*, unsigned long, "
    "unsigned long, unsigned long, unsigned long, int*, int*, int*)",
    "preprocessing_mmaSTKernel(__half*, char*, __half*, unsigned long, unsigned long, unsigned long, "
    "unsigned long, int*, int*)",
    "preprocessing_mmaSTKernel_large(__half*, char*, __half*, unsigned long, unsigned long, unsigned long, "
    "unsigned long, int*, int*)",
}

# gflags, which the reference harness includes, is not installed: this stub
# gives main.cu the few names it uses (flags keep their defaults)
GFLAGS_STUB = """#pragma once
#include <cstdint>
#include <string>
#define GFLAGS_NAMESPACE smat_gflags_stub
namespace smat_gflags_stub {
inline void ParseCommandLineFlags(int*, char***, bool) {}
inline void ShutDownCommandLineFlags() {}
}
#define DEFINE_uint32(name, val, txt) static uint32_t FLAGS_##name = (val)
#define DEFINE_bool(name, val, txt) static bool FLAGS_##name = (val)
#define DEFINE_string(name, val, txt) static std::string FLAGS_##name = (val)
"""


def test_launchers_exported_with_reference_signatures(smat_mod):
    from smat import _lib
    out = subprocess.run(["nm", "-D", "--defined-only", _lib.LIB_PATH], capture_output=True, text=True,
                         check=True).stdout
    names = [ln.split()[-1] for ln in out.splitlines() if " T " in ln]
    dem = subprocess.run(["c++filt"], input="\n".join(names), capture_output=True, text=True,
                         check=True).stdout.splitlines()
    missing = EXPECTED - set(dem)
    assert not missing, missing
    for name in _lib.REF_SHIMS:
        _lib.ref_shim(name)


def test_reference_harness_links_against_libsmat(smat_mod, oracle_lib, tmp_path):
    """The reference's benchmark driver (src/cuda_hgemm/src/main.cu with
    common/tester.h), compiled from the reference tree as it stands and linked
    against libsmat with none of the reference's mma/*.cu: every launcher it
    calls (main.cu:306-311: mmaOBTSKernel_large, mmaOBTSKernel_large_separate,
    preprocessing_mmaSTKernel_large) resolves to libsmat's. Two compile-time
    definitions stand in for the cudaDeviceProp fields CUDA 13 removed
    (clockRate, memoryClockRate, printed at main.cu:167-172); gflags is
    stubbed."""
    import os
    import shutil
    from smat import _lib
    ref = oracle_lib.reference_dir()
    if ref is None:
        pytest.skip("reference sources absent")
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(nvcc):
        pytest.skip("nvcc absent")
    src = os.path.join(ref, "src", "cuda_hgemm", "src")
    (tmp_path / "gflags").mkdir()
    (tmp_path / "gflags" / "gflags.h").write_text(GFLAGS_STUB)
    exe = tmp_path / "hgemm"
    libdir = os.path.dirname(_lib.LIB_PATH)
    cmd = [nvcc, "-std=c++17", "-gencode", "arch=compute_103a,code=sm_103a", "-w", f"-I{tmp_path}",
           f"-I{os.path.join(src, 'common')}", "-DclockRate=multiProcessorCount",
           "-DmemoryClockRate=memoryBusWidth", "-Xcompiler", "-fopenmp", os.path.join(src, "main.cu"),
           "-o", str(exe), f"-L{libdir}", "-lsmat", "-lcublas", "-lgomp", f"-Xlinker=-rpath={libdir}"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    und = subprocess.run(["nm", "-C", "-u", str(exe)], capture_output=True, text=True, check=True).stdout
    assert "mmaOBTSKernel_large" in und and "preprocessing_mmaSTKernel_large" in und
    dyn = subprocess.run(["nm", "-C", "-D", "--defined-only", _lib.LIB_PATH], capture_output=True, text=True,
                         check=True).stdout
    for ln in und.splitlines():
        name = ln.split(" U ")[-1].strip()
        if name.startswith(("mmaOBT", "mmaST", "mmaBT", "mmaCBT", "mmaT", "mmaNaive", "preprocessing_")):
            assert name in dyn, name


# ------------------------------------------------------------------------------------------------ GPU

def ref_bcsr_device(smat_mod, A, k, dev):
    """Reference-layout BCSR of A (rows padded to 16, cols to k) on the device."""
    rp, ci, v = smat_mod.csr_to_bcsr_host(A, block=(16, k))
    M = (A.rows + 15) // 16 * 16
    K = (A.cols + k - 1) // k * k
    t = lambda a: torch.from_numpy(np.ascontiguousarray(a)).to(dev)
    return t(v.reshape(-1).view(np.int16)).view(torch.float16), t(rp), t(ci), M, K, len(ci)


def fp64(A, Bh, M):
    import scipy.sparse as sps
    Asp = sps.csr_matrix((A.values.astype(np.float64), A.col_idx, A.row_ptr), shape=(A.rows, A.cols))
    r = np.zeros((M, Bh.shape[1]))
    r[: A.rows] = Asp @ Bh[: A.cols].astype(np.float64)
    return r


def rel(a, b):
    return float(np.linalg.norm(np.asarray(a, np.float64) - b) / np.linalg.norm(b))


@pytest.fixture(scope="module")
def dev():
    if not torch.cuda.is_available():
        pytest.skip("no GPU")
    return torch.device("cuda", 0)


@pytest.mark.gpu
@pytest.mark.parametrize("name,k", [("mmaOBTKernel", 16), ("mmaOBTKernel_large", 32), ("mmaOBTSKernel", 16),
                                    ("mmaOBTSKernel_large", 32)])
def test_launcher_matches_fp64(dev, smat_mod, name, k):
    from smat import _lib
    from smat import generators as G
    A = G.force_24(G.band(1000, 40, seed=2), 0.4, 16, 16, seed=3)
    v, rp, ci, M, K, nnzb = ref_bcsr_device(smat_mod, A, k, dev)
    N = 64
    Bh = np.zeros((K, N), np.float16)
    Bh[: A.cols] = np.random.default_rng(5).uniform(-1, 1, (A.cols, N)).astype(np.float16)
    Bc = torch.from_numpy(Bh).to(dev).t().contiguous()          # column-major K x N
    Cm = torch.full((M, N), float("nan"), dtype=torch.float16, device=dev)
    f = _lib.ref_shim(name)
    P = lambda t: t.data_ptr()
    for _ in range(2):                                           # first call builds, second reuses
        if "S" in name.replace("mmaOBT", "")[:1]:
            f(P(v), P(rp), P(ci), None, None, P(Bc), P(Cm), M, N, K, nnzb, None, None)
        else:
            f(P(v), P(rp), P(ci), P(Bc), P(Cm), M, N, K, nnzb, None, None)
        torch.cuda.synchronize()
        assert smat_mod.lib().smat_ref_shims_last_status() == 0, smat_mod.lib().smat_last_error()
        assert rel(Cm.float().cpu().numpy(), fp64(A, Bh, M)) <= 1e-3


@pytest.mark.gpu
def test_separate_launcher_merges_parts(dev, smat_mod):
    from smat import _lib
    from smat import generators as G
    A = G.random_block(800, 0.08, 0.3, 0.9, seed=4)
    rp, ci, v = smat_mod.csr_to_bcsr_host(A, block=(16, 32))
    M, K = (A.rows + 15) // 16 * 16, (A.cols + 31) // 32 * 32
    # split the blocks of every block row alternately into two BCSRs
    parts = [([0], [], []), ([0], [], [])]
    for r in range(len(rp) - 1):
        for j, kk in enumerate(range(rp[r], rp[r + 1])):
            p = parts[j % 2]
            p[1].append(ci[kk])
            p[2].append(v[kk])
        for p in parts:
            p[0].append(len(p[1]))
    t = lambda a, dt: torch.from_numpy(np.ascontiguousarray(np.asarray(a, dt))).to(dev)
    dv = []
    for p in parts:
        vals = np.stack(p[2]).astype(np.float16) if p[2] else np.zeros((1, 16, 32), np.float16)
        dv.append((t(vals.reshape(-1).view(np.int16), np.int16).view(torch.float16), t(p[0], np.int32),
                   t(p[1] if p[1] else [0], np.int32)))
    N = 40
    Bh = np.zeros((K, N), np.float16)
    Bh[: A.cols] = np.random.default_rng(6).uniform(-1, 1, (A.cols, N)).astype(np.float16)
    Bc = torch.from_numpy(Bh).to(dev).t().contiguous()
    Cm = torch.zeros((M, N), dtype=torch.float16, device=dev)
    P = lambda x: x.data_ptr()
    _lib.ref_shim("mmaOBTSKernel_large_separate")(P(dv[0][0]), P(dv[0][1]), P(dv[0][2]), P(dv[1][0]), P(dv[1][1]),
                                                  P(dv[1][2]), None, None, P(Bc), P(Cm), M, N, K, len(ci), None, None)
    torch.cuda.synchronize()
    assert smat_mod.lib().smat_ref_shims_last_status() == 0, smat_mod.lib().smat_last_error()
    assert rel(Cm.float().cpu().numpy(), fp64(A, Bh, M)) <= 1e-3


@pytest.mark.gpu
def test_launcher_agrees_with_reference_kernel(dev, smat_mod):
    import ref_kernel
    if not ref_kernel.available():
        pytest.skip("reference kernel not built")
    from smat import _lib
    from smat import generators as G
    A = G.band(2048, 48, seed=7)
    v, rp, ci, M, K, nnzb = ref_bcsr_device(smat_mod, A, 16, dev)
    N = 72
    Bh = np.random.default_rng(8).uniform(-1, 1, (K, N)).astype(np.float16)
    Bc = torch.from_numpy(Bh).to(dev).t().contiguous()
    Cm = torch.zeros((M, N), dtype=torch.float16, device=dev)
    _lib.ref_shim("mmaOBTKernel")(v.data_ptr(), rp.data_ptr(), ci.data_ptr(), Bc.data_ptr(), Cm.data_ptr(), M, N, K,
                                  nnzb, None, None)
    Cr, keep = ref_kernel.run(v.view(-1, 16, 16), rp, ci, M, K, Bc, N)
    torch.cuda.synchronize()
    ref = fp64(A, Bh, M)
    e_ours, e_ref = rel(Cm.float().cpu().numpy(), ref), rel(Cr.float().cpu().numpy(), ref)
    assert e_ours <= 1e-3 and rel(Cm.float().cpu().numpy(), Cr.float().cpu().numpy().astype(np.float64)) <= 1e-3
    assert e_ours <= e_ref * 1.01 + 1e-6   # FP32 accumulation is no worse than the reference's FP16


@pytest.mark.gpu
def test_preprocessing_compressor_bit_exact(dev, smat_mod, oracle_lib):
    import ref_kernel
    from smat import _lib
    from smat import generators as G
    # exact 2:4 blocks, blocks with 3 nonzeros in a group of four, -0.0 values
    A = G.force_24(G.random_block(640, 0.2, 0.2, 0.95, seed=9), 0.6, 16, 16, seed=10)
    rng = np.random.default_rng(11)
    vals = A.values.astype(np.float16)
    vals[rng.random(len(vals)) < 0.05] = np.float16(-0.0)
    M, K = (A.rows + 15) // 16 * 16, (A.cols + 15) // 16 * 16
    brp, bci, bv, info = oracle_lib.csr_to_bcsr(M, K, 16, A.row_ptr.astype(np.int32), A.col_idx, vals)
    rel_map = np.where(info != 0, np.cumsum(info != 0) - 1, -1).astype(np.int32)
    assert (info == 1).sum() > 10
    t = lambda a: torch.from_numpy(np.ascontiguousarray(a)).to(dev)
    dv = t(bv.reshape(-1).view(np.int16)).view(torch.float16)
    dinfo, drel = t(info.astype(np.int32)), t(rel_map)
    nnzb = len(bci)
    outs = []
    for which in ("ours", "ref"):
        meta = torch.full((nnzb * 32,), 0x5A, dtype=torch.int8, device=dev)      # untouched blocks keep this
        sp = torch.full((nnzb * 128,), 7.0, dtype=torch.float16, device=dev)
        if which == "ours":
            _lib.ref_shim("preprocessing_mmaSTKernel")(dv.data_ptr(), meta.data_ptr(), sp.data_ptr(), M, 64, K, nnzb,
                                                       dinfo.data_ptr(), drel.data_ptr())
        else:
            if not ref_kernel.compress_available():
                continue
            keep = ref_kernel.compress24(dv, dinfo, drel, M, 64, K, meta, sp)
        torch.cuda.synchronize()
        outs.append((meta.cpu().numpy(), sp.cpu().numpy().view(np.uint16)))
    if len(outs) < 2:
        pytest.skip("reference compressor not built")
    m0, s0 = outs[0]
    m1, s1 = outs[1]
    assert np.array_equal(m0, m1)
    assert np.array_equal(s0, s1)


def ref_labels_and_map(oracle_lib, A, k, vals=None):
    """The reference's BCSR of A with k-wide blocks (oracle csrToBcsr), its
    blockInfo labels and relativeBlockIndexMapping (block-grid cell -> block)."""
    vals = A.values.astype(np.float16) if vals is None else vals
    M, K = (A.rows + 15) // 16 * 16, (A.cols + k - 1) // k * k
    # the row pointer covers the padded rows (csrToBcsr reads M + 1 entries)
    rp = np.concatenate([A.row_ptr, np.full(M - A.rows, A.row_ptr[-1])]).astype(np.int32)
    brp, bci, bv, info = oracle_lib.csr_to_bcsr(M, K, k, rp, A.col_idx, vals)
    rel_map = np.where(info != 0, np.cumsum(info != 0) - 1, -1).astype(np.int32)
    return M, K, brp, bci, bv, info, rel_map


@pytest.mark.gpu
def test_preprocessing_large_compressor_bit_exact(dev, smat_mod, oracle_lib):
    """preprocessing_mmaSTKernel_large against the reference's own compressor
    (mmaST_large.cu:22-152, built from its source), bit for bit: values and
    every metadata byte, blocks it does not write included."""
    import ref_kernel
    from smat import _lib
    from smat import generators as G
    A = G.force_24(G.random_block(704, 0.2, 0.2, 0.95, seed=19), 0.6, 16, 16, seed=20)
    rng = np.random.default_rng(21)
    vals = A.values.astype(np.float16)
    vals[rng.random(len(vals)) < 0.05] = np.float16(-0.0)
    M, K, brp, bci, bv, info, rel_map = ref_labels_and_map(oracle_lib, A, 32, vals)
    assert (info == 1).sum() > 10
    t = lambda a: torch.from_numpy(np.ascontiguousarray(a)).to(dev)
    dv = t(bv.reshape(-1).view(np.int16)).view(torch.float16)
    dinfo, drel = t(info.astype(np.int32)), t(rel_map)
    nnzb = len(bci)
    outs = []
    for which in ("ours", "ref"):
        meta = torch.full((nnzb * 64,), 0x5A, dtype=torch.int8, device=dev)      # bytes not written keep this
        sp = torch.full((nnzb * 256,), 7.0, dtype=torch.float16, device=dev)
        if which == "ours":
            _lib.ref_shim("preprocessing_mmaSTKernel_large")(dv.data_ptr(), meta.data_ptr(), sp.data_ptr(), M, 64, K,
                                                             nnzb, dinfo.data_ptr(), drel.data_ptr())
        else:
            if not ref_kernel.compress_large_available():
                continue
            keep = ref_kernel.compress24(dv, dinfo, drel, M, 64, K, meta, sp, large=True)
        torch.cuda.synchronize()
        outs.append((meta.cpu().numpy(), sp.cpu().numpy().view(np.uint16)))
    if len(outs) < 2:
        pytest.skip("reference compressor not built")
    (m0, s0), (m1, s1) = outs
    assert np.array_equal(s0, s1)
    assert np.array_equal(m0, m1), np.nonzero(m0 != m1)[0][:16]


@pytest.mark.gpu
def test_harness_sparse24_2_large_flow(dev, smat_mod, oracle_lib):
    """What tester.h:461-504 (evaluateSparse24_2) does with the launchers
    main.cu:306-308 passes: preprocessing_mmaSTKernel_large on the full BCSR,
    then mmaOBTSKernel_large with its metadata and values, blockInfo and the
    relative block map; C against FP64 (1e-3, FP16 C)."""
    from smat import _lib
    from smat import generators as G
    A = G.force_24(G.rmat(11, 30000, seed=12), 0.3, 16, 16, seed=13)
    M, K, brp, bci, bv, info, rel_map = ref_labels_and_map(oracle_lib, A, 32)
    t = lambda a: torch.from_numpy(np.ascontiguousarray(a)).to(dev)
    dv = t(bv.reshape(-1).view(np.int16)).view(torch.float16)
    drp, dci, dinfo, drel = t(brp), t(bci), t(info.astype(np.int32)), t(rel_map)
    nnzb = len(bci)
    N = 128
    Bh = np.zeros((K, N), np.float16)
    Bh[: A.cols] = np.random.default_rng(14).uniform(-1, 1, (A.cols, N)).astype(np.float16)
    Bc = torch.from_numpy(Bh).to(dev).t().contiguous()
    meta = torch.zeros((nnzb * 64,), dtype=torch.int8, device=dev)
    sp = torch.zeros((nnzb * 256,), dtype=torch.float16, device=dev)
    Cm = torch.full((M, N), float("nan"), dtype=torch.float16, device=dev)
    P = lambda x: x.data_ptr()
    _lib.ref_shim("preprocessing_mmaSTKernel_large")(P(dv), P(meta), P(sp), M, N, K, nnzb, P(dinfo), P(drel))
    torch.cuda.synchronize()
    for _ in range(2):
        _lib.ref_shim("mmaOBTSKernel_large")(P(dv), P(drp), P(dci), P(meta), P(sp), P(Bc), P(Cm), M, N, K, nnzb,
                                             P(dinfo), P(drel))
        torch.cuda.synchronize()
        assert smat_mod.lib().smat_ref_shims_last_status() == 0, smat_mod.lib().smat_last_error()
        e = rel(Cm.float().cpu().numpy(), fp64(A, Bh, M))
        print(f"evaluateSparse24_2 flow: rel err vs FP64 {e:.2e}")
        assert e <= 1e-3


@pytest.mark.gpu
def test_harness_split_large_flow(dev, smat_mod, oracle_lib):
    """What tester.h:554-590 (evaluateSplit) does: mmaOBTSKernel_large_separate
    with the full BCSR's values passed for both parts, the 2:4 and dense row
    pointers / column starts of filterBcsrBlocks, and the relative block map
    through which the reference kernel finds each block's values; C against
    FP64 over all blocks (the reference's own kernel skips the 2:4 part)."""
    from smat import _lib
    from smat import generators as G
    A = G.force_24(G.band(1500, 70, seed=15), 0.4, 16, 16, seed=16)
    M, K, brp, bci, bv, info, rel_map = ref_labels_and_map(oracle_lib, A, 32)
    (rp24, ci24, _), (rpd, cid, _), grid = smat_mod.csr_to_bcsr_split_host(A, block_cols=32)
    assert np.array_equal(grid.reshape(-1), info)
    assert len(ci24) > 0 and len(cid) > 0
    t = lambda a: torch.from_numpy(np.ascontiguousarray(a)).to(dev)
    dv = t(bv.reshape(-1).view(np.int16)).view(torch.float16)
    d = [t(x if len(x) else np.zeros(1, np.int32)) for x in (rp24, ci24, rpd, cid)]
    dinfo, drel = t(info.astype(np.int32)), t(rel_map)
    N = 64
    Bh = np.zeros((K, N), np.float16)
    Bh[: A.cols] = np.random.default_rng(17).uniform(-1, 1, (A.cols, N)).astype(np.float16)
    Bc = torch.from_numpy(Bh).to(dev).t().contiguous()
    Cm = torch.full((M, N), float("nan"), dtype=torch.float16, device=dev)
    P = lambda x: x.data_ptr()
    _lib.ref_shim("mmaOBTSKernel_large_separate")(P(dv), P(d[0]), P(d[1]), P(dv), P(d[2]), P(d[3]), None, None,
                                                  P(Bc), P(Cm), M, N, K, len(bci), P(dinfo), P(drel))
    torch.cuda.synchronize()
    assert smat_mod.lib().smat_ref_shims_last_status() == 0, smat_mod.lib().smat_last_error()
    e = rel(Cm.float().cpu().numpy(), fp64(A, Bh, M))
    print(f"evaluateSplit flow: rel err vs FP64 {e:.2e}")
    assert e <= 1e-3
