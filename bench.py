"""SpMM benchmark on one GB300 (one JSON line on stdout).

Workload (the R-MAT configuration): R-MAT 2^16 x 2^16 (a=0.57, b=c=0.19,
d=0.05), 2,000,000 distinct entries, rows randomly permuted, FP16 N(0,1)
values; Jaccard row reordering (Keeper, tau = 0.6, 16-column blocks,
16-row groups, fixed-size regrouping); 16 x 16 BCSR; 30 % of the nonzero
blocks rewritten to an exact 2:4 pattern; B 65536 x 128 FP16 U[-1,1] in the
reference's column-major layout; FP32 accumulation, FP32 C in the original
row order. All data synthetic and seeded.

A step is one SpMM C = A * B with A (BCSR), B and C resident on the device.
`value` is useful TFLOP/s (2 * nnz * N / t); `e2e` is the same metric
through smat_spmm_host with B copied in from pinned host memory and C copied
back every step. The matrix A (~0.4 GB) is larger than L2 (129 MB), so no
L2 flush is done between steps.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl smat|reference]

`--impl reference` times the reference's CPU SpMM (CSR::multiply,
preprocess/src/general/csr.cpp:47-63, restated in oracle/) on the host cores
on bounded row samples of the same matrix.
"""
from __future__ import annotations

import argparse
import hashlib
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(ROOT, "sptc-smat_gb300"))

METRIC = "SpMM useful TFLOP/s, chosen form vs plain FP16 BCSR on one GB300 at stated rel err"

WORKLOAD = {
    "workload": "rmat16_2M_reordered_tau0.6_bcsr16x16_24frac0.3_N128",
    "generator": "R-MAT 2^16, a=0.57 b=c=0.19 d=0.05, 2.0M unique, rows permuted, FP16 N(0,1)",
    "reorder": "Keeper (-a 5), tau=0.6, col_block=16, row_block=16, fixed size (-F 1)",
    "block": [16, 16],
    "forced_24_fraction": 0.3,
    "N": 128,
    "B": "65536x128 FP16 U[-1,1], column-major",
    "C": "FP32, original row order",
    "form": "plain FP16 (tcgen05 kind::f16, FP32 accumulate)",
    "l2": "no flush: A (~0.4 GB) is larger than the 129 MB L2",
    "step": "pack B into 4 KB tiles + tensor-core SpMM (2 launches), replayed as one captured CUDA graph",
}


def log(*a):
    print(*a, file=sys.stderr, flush=True)


# ---------------------------------------------------------------------------------------------- workload

def build_matrix():
    """(A in original row order, perm) for the R-MAT workload (smat.workloads.rmat16; the reorder is cached on
    disk)."""
    from smat import workloads

    t0 = time.time()
    A, perm = workloads.rmat16()
    log(f"[bench] matrix ready in {time.time() - t0:.1f}s: nnz={A.nnz}")
    return A, perm


def workload_config(A, world):
    """The `config` of the R-MAT line, identical in both arms."""
    return dict(WORKLOAD, nnz=int(A.nnz), parallelism=f"replicas x{world}" if world > 1 else "single GPU")


# ---------------------------------------------------------------------------------------------- clocks

class ClockSampler:
    """nvidia-smi clock / throttle sampling during the timed region."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, device_index: int):
        self.dev = device_index
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.dev), f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "100"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.th = threading.Thread(target=self._read, daemon=True)
            self.th.start()
        except OSError:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        self.th.join(timeout=2)
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx = float(f[2])
            except ValueError:
                continue
            for nm, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": mx, "reasons": sorted(reasons),
                "samples": len(sm)}


# ---------------------------------------------------------------------------------------------- arms

def peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def profile_traffic():
    """DRAM bytes per launch of the SpMM kernel from the committed ncu summary, if present."""
    p = os.path.join(ROOT, "profiles", "spmm_tc_rmat16_traffic.json")
    if os.path.exists(p):
        with open(p) as f:
            return json.load(f)
    return None


def cpu_baseline(A, N, threads=1, budget_s=12.0, max_rows=None):
    """CSR::multiply (restated, oracle/) over a bounded row sample; returns (useful TFLOP/s, sample text)."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import concurrent.futures as cf

    import oracle as O
    O.lib()
    rows = A.rows
    rp = A.row_ptr.astype(np.int64)
    ci = A.col_idx.astype(np.int64)
    v = A.values.astype(np.float32)
    rng = np.random.default_rng(0)
    Bc = rng.uniform(-1, 1, rows * N).astype(np.float32)
    Cc = np.zeros(rows * N, np.float32)
    # calibrate on a small prefix
    r_cal = min(rows, 256)
    t = time.perf_counter()
    O.csr_multiply_f32_range(rows, 0, r_cal, rp, ci, v, Bc, N, Cc)
    dt = max(time.perf_counter() - t, 1e-6)
    per_nnz = dt / max(int(rp[r_cal]), 1)
    target_nnz = budget_s / per_nnz * threads
    r1 = int(np.searchsorted(rp, target_nnz))
    r1 = max(1, min(rows, r1 if max_rows is None else min(r1, max_rows)))
    # row ranges with equal nonzero counts (R-MAT rows differ by orders of
    # magnitude, so equal row counts would leave one thread with the hubs)
    bounds = np.searchsorted(rp, np.linspace(0, int(rp[r1]), threads + 1)).astype(np.int64)
    bounds[0], bounds[-1] = 0, r1
    t = time.perf_counter()
    with cf.ThreadPoolExecutor(max_workers=threads) as ex:
        list(ex.map(lambda k: O.csr_multiply_f32_range(rows, int(bounds[k]), int(bounds[k + 1]), rp, ci, v, Bc, N,
                                                       Cc), range(threads)))
    dt = time.perf_counter() - t
    nnz = int(rp[r1])
    return 2.0 * nnz * N / dt / 1e12, f"rows 0..{r1} of {rows} ({nnz} of {A.nnz} nnz), N={N}, {dt:.2f}s"


def dist_init(args):
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    pg = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("gloo")
        pg = dist
    return world, rank, local, pg


def run_reference(args):
    world, rank, local, pg = dist_init(args)
    if rank != 0:
        if pg:
            pg.barrier()
        return
    A, _ = build_matrix()
    N = WORKLOAD["N"]
    threads = os.cpu_count() or 1
    vals = []
    sample = ""
    for _ in range(args.warmup):
        cpu_baseline(A, N, threads=threads, budget_s=1.0)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        v, sample = cpu_baseline(A, N, threads=threads, budget_s=max(2.0, 60.0 / max(args.steps, 1)))
        vals.append(v)
    wall = time.perf_counter() - t0
    value = float(np.mean(vals))
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": "TFLOP/s", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": wall / max(args.steps, 1) * 1e3,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic", "config": workload_config(A, world),
            "cpu_baseline": {"value": value, "unit": "TFLOP/s", "cores": threads, "kind": "port",
                             "sample": sample + "; reference CSR::multiply loop (csr.cpp:47-63), row ranges on "
                                                f"{threads} threads"},
            "e2e": {"value": value, "unit": "TFLOP/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)
    if pg:
        pg.barrier()


REORDER_WORKLOAD = {
    "workload": "rmat16_2M_reorder_tau0.6",
    "generator": "R-MAT 2^16, a=0.57 b=c=0.19 d=0.05, 2.0M unique, rows permuted",
    "reorder": "Keeper (-a 5), tau=0.6, col_block=16, row_block=16, fixed size (-F 1)",
}


def run_reorder(args):
    """The reorder step alone on the R-MAT pattern: smat_reorder (this
    library, host cores), or with --impl reference the reference's own
    BlockingEngine built from its sources (oracle/_ref, single-threaded as
    the reference runs it), where that build exists. Seconds per reorder,
    and the permutation's hash so that the two arms can be compared."""
    import smat
    from smat import generators as G
    A0 = G.rmat(16, 2_000_000, seed=3)
    times, perm, extra = [], None, {}
    for _ in range(max(args.steps, 1)):
        t = time.perf_counter()
        if args.impl == "reference":
            sys.path.insert(0, os.path.join(ROOT, "oracle"))
            import oracle as O
            if not O.ref_available():
                print(json.dumps({"impl": "reference", "workload": REORDER_WORKLOAD["workload"],
                                  "unavailable": "the reference preprocess library is built only where the "
                                                 "reference sources are (oracle/Makefile)"}), flush=True)
                return
            perm, _, st = O.ref_reorder(A0.row_ptr, A0.col_idx, A0.cols, 0.6, 16, 16)
            extra = {"comparisons": int(st[0]), "merges": int(st[1]), "cores": 1}
        else:
            r = smat.reorder(A0, tau=0.6, col_block=16, row_block=16, algo=5, force_fixed=True,
                             use_gpu=args.reorder_gpu)
            perm = r.perm
            extra = {"comparisons": int(r.comparisons), "merges": int(r.merges), "cores": os.cpu_count(),
                     "distances_on": "GPU (seed loop and commits on the host)" if args.reorder_gpu else "host cores"}
        times.append(time.perf_counter() - t)
    line = {"metric": "reorder seconds", "value": float(np.median(times)), "unit": "s", "steps": len(times),
            "higher_is_better": False, "data": "synthetic", "config": REORDER_WORKLOAD,
            "perm_sha1": hashlib.sha1(np.ascontiguousarray(perm, np.int64).tobytes()).hexdigest()[:16]} | extra
    if args.impl == "reference":
        line["impl"] = "reference"
    print(json.dumps(line), flush=True)


TILES_WORKLOAD = {
    "workload": "rmat16_reordered_tiles4x4",
    "source": "the R-MAT workload's reordered BCSR (tau 0.6, 30 % of blocks forced to 2:4)",
    "step": "smat_tiles_create: device BCSR -> the reference's merged 4 x 4-block tiles (synchronous)",
    "spmm": "mmaOBTKernel_tiled / mmaOBTSKernel_tiled_large on the merged arrays, N = 128, FP16 B (column-major) "
            "and C, legacy default stream",
}


def run_tiles(args):
    """The merged 4 x 4-block tiles of the reference's bcsrBlocking
    (matrix.h:794-1137) built on the GPU from the R-MAT workload's BCSR, at
    16 x 16 and 16 x 32 blocks: seconds per build (wall clock: the build
    synchronises), checked bit for bit against the oracle's host build (also
    timed, one thread), and the `_tiled` launcher's SpMM on the result
    (CUDA events) with its error against FP64 on a row sample."""
    import scipy.sparse as sps
    import torch

    import smat
    from smat import _lib
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as O
    dev = torch.device("cuda", 0)
    A, perm = build_matrix()
    N = 128
    rng = np.random.default_rng(2)
    for k in (16, 32):
        brp, bci, bv = smat.csr_to_bcsr_host(A, block=(16, k), row_perm=perm)
        M, K = (A.rows + 15) // 16 * 16, (A.cols + k - 1) // k * k
        up = lambda a: torch.from_numpy(np.ascontiguousarray(a)).to(dev)
        drp, dci, dv = up(brp), up(bci), up(bv.reshape(-1).view(np.int16))
        torch.cuda.synchronize()
        times, T = [], None
        for i in range(args.warmup + args.steps):
            if T is not None:
                T.close()
            t0 = time.perf_counter()
            T = smat.Tiles(M, K, k, drp, dci, dv)
            dt = time.perf_counter() - t0
            if i >= args.warmup:
                times.append(dt)
        got = T.to_host()
        t0 = time.perf_counter()
        want = O.bcsr_blocking(M, K, k, brp, bci, bv)
        t_host = time.perf_counter() - t0
        exact = all(np.array_equal(got[x].reshape(-1), want[x].reshape(-1)) for x in O.TILE_KEYS)
        del want
        # the _tiled launcher on the merged arrays (C rows in the reordered order)
        Bh = np.zeros((K, N), np.float16)
        Bh[: A.cols] = rng.uniform(-1, 1, (A.cols, N)).astype(np.float16)
        Bc = torch.from_numpy(Bh).to(dev).t().contiguous()
        Cm = torch.empty((M, N), dtype=torch.float16, device=dev)
        d = T.desc
        name = "mmaOBTKernel_tiled" if k == 16 else "mmaOBTSKernel_tiled_large"
        f = _lib.ref_shim(name)

        def call():
            if k == 16:
                f(d.values, d.row_ptr, d.col_idx, Bc.data_ptr(), Cm.data_ptr(), M, N, K, len(bci), d.block_info,
                  d.rel_map)
            else:
                f(d.values, d.row_ptr, d.col_idx, None, None, Bc.data_ptr(), Cm.data_ptr(), M, N, K, len(bci),
                  d.block_info, d.rel_map, d.tile_info)

        for _ in range(max(args.warmup, 1)):
            call()
        torch.cuda.synchronize()
        st = smat.lib().smat_ref_shims_last_status()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        for _ in range(args.steps):
            call()
        e1.record()
        torch.cuda.synchronize()
        ms = e0.elapsed_time(e1) / max(args.steps, 1)
        rows = np.sort(rng.choice(A.rows, min(4096, A.rows), replace=False))
        src = perm[rows]
        Asp = sps.csr_matrix((A.values.astype(np.float64), A.col_idx, A.row_ptr), shape=(A.rows, A.cols))
        ref = Asp[src] @ Bh[: A.cols].astype(np.float64)
        Cs = Cm.float().cpu().numpy()[rows].astype(np.float64)
        err = float(np.linalg.norm(Cs - ref) / np.linalg.norm(ref))
        smat.lib().smat_ref_shims_release()
        print(json.dumps({
            "metric": "merged-tile build seconds", "value": float(np.median(times)), "unit": "s",
            "higher_is_better": False, "steps": len(times), "warmup": args.warmup, "data": "synthetic",
            "config": dict(TILES_WORKLOAD, block=[16, k]), "nnzb": int(len(bci)), "n_tiles": int(T.n_tiles),
            "n_rowptr": int(T.n_rowptr), "bit_exact_vs_oracle": bool(exact),
            "cpu_baseline": {"value": t_host, "unit": "s", "cores": 1, "kind": "port",
                             "sample": "whole matrix; the oracle's restatement of bcsrBlocking (map lookup in "
                                       "place of the reference's linear search over the tiles made so far)"},
            "tiled_spmm": {"launcher": name, "ms": ms, "status": int(st),
                           "useful_tflops": 2.0 * A.nnz * N / (ms * 1e-3) / 1e12,
                           "rel_err_vs_fp64_4096_rows": err},
        }), flush=True)
        T.close()


def run_smat(args):
    import torch

    import smat
    world, rank, local, pg = dist_init(args)
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    A, perm = build_matrix()
    N = WORKLOAD["N"]
    t0 = time.time()
    M = smat.Bcsr(A, block=(16, 16), forms=(smat.FORM_F16,), row_perm=perm, device=local)
    log(f"[bench] BCSR built in {time.time() - t0:.1f}s: {M.info}")
    info = M.info
    rng = np.random.default_rng(2)
    Bh = rng.uniform(-1, 1, (A.cols, N)).astype(np.float16)
    B = torch.from_numpy(Bh).to(dev).t().contiguous().t()        # column-major (K, N)
    Cd = torch.empty((A.rows, N), dtype=torch.float32, device=dev)
    stream = torch.cuda.Stream(device=dev)
    sp = stream.cuda_stream
    ws_bytes = M.workspace_size(smat.FORM_F16, smat.F16, N)
    ws = torch.empty(ws_bytes, dtype=torch.uint8, device=dev)

    def step():
        M.spmm_raw(smat.FORM_F16, B, smat.F16, smat.COL_MAJOR, A.cols, Cd, smat.F32, N, N, ws, ws_bytes, sp)

    # correctness of this exact configuration against an FP64 product (scipy, independent of the oracle)
    step()
    torch.cuda.synchronize(dev)
    M.check_device_error()
    import scipy.sparse as sps
    Asp = sps.csr_matrix((A.values.astype(np.float64), A.col_idx, A.row_ptr), shape=(A.rows, A.cols))
    ref = Asp @ Bh.astype(np.float64)       # kept for the other forms and the 2:4 path
    ref_nrm = float(np.linalg.norm(ref))
    got = Cd.cpu().numpy().astype(np.float64)
    rel_err = float(np.linalg.norm(got - ref) / ref_nrm)
    log(f"[bench] rel Frobenius error vs FP64: {rel_err:.3e}")
    del got

    for _ in range(max(args.warmup, 3)):
        step()
    torch.cuda.synchronize(dev)
    # the step (work-counter memset, B packing, contraction) captured once as
    # a CUDA graph and replayed: the library's calls are capture-safe
    graph = torch.cuda.CUDAGraph()
    with torch.cuda.graph(graph, stream=stream):
        step()
    with torch.cuda.stream(stream):
        for _ in range(2):
            graph.replay()
    torch.cuda.synchronize(dev)
    M.check_device_error()
    clocks = ClockSampler(local)
    clocks.start()
    time.sleep(0.3)
    if pg:
        pg.barrier()
    torch.cuda.synchronize(dev)
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with torch.cuda.stream(stream):
        ev0.record(stream)
        for _ in range(args.steps):
            graph.replay()
        ev1.record(stream)
    torch.cuda.synchronize(dev)
    ms_total = ev0.elapsed_time(ev1)
    # per-launch durations of the two kernels on the launching stream: the B
    # packing and the tensor-core contraction (the roofline's kernel)
    evs = [[torch.cuda.Event(enable_timing=True) for _ in range(3)] for _ in range(args.steps)]
    for a, b, c in evs:
        a.record(stream)
        M.pack_b(smat.FORM_F16, B, smat.F16, smat.COL_MAJOR, A.cols, N, ws, ws_bytes, sp)
        b.record(stream)
        M.spmm_packed(smat.FORM_F16, ws, N, Cd, smat.F32, N, sp)
        c.record(stream)
    torch.cuda.synchronize(dev)
    clk = clocks.stop()
    pack_ms = float(np.mean([a.elapsed_time(b) for a, b, c in evs]))
    kern_ms = float(np.mean([b.elapsed_time(c) for a, b, c in evs]))
    ms = ms_total / args.steps
    if pg:
        import torch.distributed as dist
        t = torch.tensor([ms, kern_ms], dtype=torch.float64)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        ms, kern_ms = float(t[0]), float(t[1])

    # the same step with the structured-sparse path on: exact-2:4 blocks on
    # tcgen05.mma.sp (second launch), the others on the dense kernel
    sp24 = []
    for unit_min in ([] if args.no_sp24 else [1, 8]):
        M24 = smat.Bcsr(A, block=(16, 16), forms=(smat.FORM_F16,), row_perm=perm, device=local, use_24=unit_min)
        ws24_bytes = M24.workspace_size(smat.FORM_F16, smat.F16, N)
        ws24 = torch.empty(ws24_bytes, dtype=torch.uint8, device=dev)
        C24 = torch.empty((A.rows, N), dtype=torch.float32, device=dev)

        def step24():
            M24.spmm_raw(smat.FORM_F16, B, smat.F16, smat.COL_MAJOR, A.cols, C24, smat.F32, N, N, ws24, ws24_bytes, sp)

        step24()
        torch.cuda.synchronize(dev)
        M24.check_device_error()
        got24 = C24.cpu().numpy().astype(np.float64)
        err24 = float(np.linalg.norm(got24 - ref) / ref_nrm)
        del got24
        for _ in range(max(args.warmup, 3)):
            step24()
        g24 = torch.cuda.CUDAGraph()
        with torch.cuda.graph(g24, stream=stream):
            step24()
        with torch.cuda.stream(stream):
            g24.replay()
        torch.cuda.synchronize(dev)
        f0, f1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        with torch.cuda.stream(stream):
            f0.record(stream)
            for _ in range(args.steps):
                g24.replay()
            f1.record(stream)
        torch.cuda.synchronize(dev)
        M24.check_device_error()
        ms24 = f0.elapsed_time(f1) / args.steps
        i24 = M24.info
        # 2:4 blocks move 256 B of kept values + 32 B of metadata instead of 512 B
        n24 = i24["n_blocks_24"]
        sp24.append({"unit_min_blocks": unit_min,
                "value": world * 2.0 * A.nnz * N / (ms24 * 1e-3) / 1e12, "unit": "TFLOP/s", "ms_per_step": ms24,
                "n_blocks_24": n24, "nnzb": i24["nnzb"], "rel_err_vs_fp64": err24,
                "a_bytes": (i24["nnzb"] - n24) * 512 + n24 * 288, "a_bytes_dense_path": i24["nnzb"] * 512,
                "step": "pack B (4 KB tiles, then 8 KB 2:4 windows) + dense SpMM over the other blocks + "
                        "tcgen05.mma.sp over the routed exact-2:4 blocks (4 launches), one CUDA graph"})
        log(f"[bench] 2:4 path (units of >= {unit_min}): {n24} of {i24['nnzb']} blocks on mma.sp, "
            f"{ms24:.4f} ms/step, rel err {err24:.3e}")
        M24.close()
        del ws24, C24

    # the metric's comparison: every precision form on the same matrix and B
    # (one BCSR per form, default shape, eager steps), each with its error
    # against the FP64 product and its bound; the chosen form is the fastest
    # within its bound
    forms = []
    if not args.no_forms:
        for name, f in FORM_BOUNDS_ORDER:
            fid = getattr(smat, f)
            # plain FP16 is timed again the same way as the others (eager steps)
            Mf = M if name == "f16" else smat.Bcsr(A, block=(16, 16), forms=(fid,), row_perm=perm, device=local)
            wsf_bytes = Mf.workspace_size(fid, smat.F16, N)
            wsf = torch.empty(wsf_bytes, dtype=torch.uint8, device=dev)
            Cf = torch.empty((A.rows, N), dtype=torch.float32, device=dev)

            def stepf():
                Mf.spmm_raw(fid, B, smat.F16, smat.COL_MAJOR, A.cols, Cf, smat.F32, N, N, wsf, wsf_bytes, sp)

            stepf()
            torch.cuda.synchronize(dev)
            Mf.check_device_error()
            errf = float(np.linalg.norm(Cf.cpu().numpy().astype(np.float64) - ref) / ref_nrm)
            for _ in range(max(args.warmup, 3)):
                stepf()
            torch.cuda.synchronize(dev)
            g0, g1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            g0.record(stream)
            for _ in range(args.steps):
                stepf()
            g1.record(stream)
            torch.cuda.synchronize(dev)
            Mf.check_device_error()
            msf = g0.elapsed_time(g1) / args.steps
            forms.append(dict(form=name, value=None, ms_per_step=msf, rel_err_vs_fp64=errf,
                              bound=FORM_BOUNDS[name], a_bytes=FORM_A_BYTES[name]))
            log(f"[bench] form {name}: {msf:.4f} ms/step, rel err {errf:.3e}")
            if Mf is not M:
                Mf.close()
            del wsf, Cf
    del ref

    # e2e through the host-buffer entry point: pinned B in, C out, every step
    Bhost = torch.empty((N, A.cols), dtype=torch.float16).pin_memory()
    Bhost.copy_(torch.from_numpy(np.ascontiguousarray(Bh.T)))
    Chost = torch.empty((A.rows, N), dtype=torch.float32).pin_memory()
    bview = Bhost.numpy().T                                           # (K, N), Fortran order
    cview = Chost.numpy()

    def step_host():
        M.spmm_host(bview, smat.FORM_F16, np.float32, out=cview, stream=sp)

    for _ in range(2):
        step_host()
    torch.cuda.synchronize(dev)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(args.steps):
        step_host()
    e1.record(stream)
    torch.cuda.synchronize(dev)
    e2e_ms = e0.elapsed_time(e1) / args.steps
    if pg:
        import torch.distributed as dist
        t = torch.tensor([e2e_ms], dtype=torch.float64)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        e2e_ms = float(t[0])

    nnz, nnzb = A.nnz, info["nnzb"]
    useful = 2.0 * nnz * N
    stored = 2.0 * nnzb * 256 * N
    value = world * useful / (ms * 1e-3) / 1e12
    nbr = info["rows_padded"] // 16
    # contraction kernel, BCSR minimum: FP16 block values + one 4-byte column index per block + block-row
    # pointers, B once (FP16, packed) and C once (FP32)
    alg_bytes = nnzb * (256 * 2 + 4) + (nbr + 1) * 4 + A.cols * N * 2 + A.rows * N * 4
    peak, peak_kind = peaks()
    achieved = alg_bytes / (kern_ms * 1e-3) / 1e9
    tr = profile_traffic()
    # the contraction's staging traffic through L2: every stage's A region
    # (blocks + MMA list) and one 4 KB B tile per distinct block column of a
    # panel (n_union_cols per 128-column pass)
    staged = nnzb * 512 + info["n_union_cols"] * 4096 * ((N + 127) // 128)
    line = {
        "metric": METRIC, "value": value, "unit": "TFLOP/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f16", "data": "synthetic",
        "config": workload_config(A, world),
        "matrix": {"nnzb": nnzb, "fill": info["fill"], "n_union_cols": info["n_union_cols"],
                   "n_blocks_24": info["n_blocks_24"], "panel_rows": info["panel_rows"]},
        "rel_err_vs_fp64": rel_err,
        "stored_tflops": world * stored / (ms * 1e-3) / 1e12,
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": achieved / peak, "peak_kind": f"{peak_kind} hbm_gbs",
                     "traffic": (tr["dram_bytes_per_launch"] if tr else None),
                     "traffic_source": (tr["source"] if tr else None),
                     "algorithmic_bytes_per_launch": alg_bytes, "kernel": "spmm_tc_kernel",
                     "kernel_ms": kern_ms, "pack_b_ms": pack_ms},
        "staging": {"bytes_per_launch": staged, "achieved_gbs": staged / (kern_ms * 1e-3) / 1e9,
                    "bytes_per_clk_per_sm": staged / (kern_ms * 1e-3) / 152 / (clk["sm_mhz"] * 1e6)
                    if clk.get("sm_mhz") else None,
                    "note": "what the stages pull from L2 into shared memory: every A block once plus one 4 KB B "
                            "tile per distinct block column of a 16-row panel (ncu: 1.86 GB L2->SM per launch); "
                            "the roofline above counts B once"},
        "clocks": clk,
        "e2e": {"value": world * useful / (e2e_ms * 1e-3) / 1e12, "unit": "TFLOP/s",
                "h2d_bytes_per_step": A.cols * N * 2, "d2h_bytes_per_step": A.rows * N * 4, "ms_per_step": e2e_ms},
        "gpu_launches": 2 * args.steps,
    }
    if sp24:
        line["sp24_path"] = sp24
    if forms:
        for fm in forms:
            fm["value"] = world * useful / (fm["ms_per_step"] * 1e-3) / 1e12
            fb = nnzb * (fm["a_bytes"] + 4) + (nbr + 1) * 4 + A.cols * N * 2 + A.rows * N * 4
            fm["roofline_frac_step"] = fb / (fm["ms_per_step"] * 1e-3) / 1e9 / peak
            fm["within_bound"] = fm["rel_err_vs_fp64"] <= fm["bound"]
        ok = [fm for fm in forms if fm["within_bound"]]
        best = max(ok, key=lambda fm: fm["value"]) if ok else None
        plain = forms[0]
        line["forms"] = {
            "per_form": forms,
            "chosen": best["form"] if best else None,
            "chosen_vs_plain_f16": (best["value"] / plain["value"]) if best else None,
            "note": "useful TFLOP/s of each form's step (pack B + contraction, eager launches) on this matrix "
                    "and B (FP16 B, FP32 C), error vs the FP64 product and the form's bound (BF16 held to plain "
                    "FP16's); roofline_frac_step = the form's BCSR-minimum bytes over its step time, of measured "
                    "HBM",
        }
    if rank == 0:
        cpu_v, sample = cpu_baseline(A, N, threads=1, budget_s=12.0)
        line["cpu_baseline"] = {"value": cpu_v, "unit": "TFLOP/s", "cores": 1, "kind": "port",
                                "sample": sample + "; CSR::multiply loop (csr.cpp:47-63), 1 thread"}
        print(json.dumps(line), flush=True)
    if pg:
        pg.barrier()
    M.close()


# forms of the metric's comparison: (name, smat attribute), their error
# bounds against FP64 and the bytes of one 16 x 16 block of A
# (BF16 has no bound of its own in the metric: it is held to plain FP16's)
FORM_BOUNDS_ORDER = [("f16", "FORM_F16"), ("bf16", "FORM_BF16"), ("fp8", "FORM_FP8"),
                     ("split_bf16", "FORM_SPLIT_BF16")]
FORM_BOUNDS = {"f16": 1e-3, "bf16": 1e-3, "fp8": 2e-2, "split_bf16": 1e-3}
FORM_A_BYTES = {"f16": 512, "bf16": 512, "fp8": 260, "split_bf16": 1024}

FORMS_WORKLOAD = {
    "workload": "stencil27_64cubed_N256",
    "generator": "27-point stencil on a 64^3 grid, natural order, off-diagonal N(1,0.1), diagonal 27+N(0,1), FP32",
    "block": [16, 16],
    "N": 256,
    "B": "262144x256 FP32 N(0,1), row-major",
    "C": "FP32",
    "l2": "no flush: B (268 MB FP32) and C (268 MB) exceed the 129 MB L2",
}


def run_forms(args):
    """The precision forms on the stencil workload: per form one JSON line
    with the default tile shape and one with the shape smat_autotune measured
    fastest for it (panel rows x split threshold x N-tile width x pipeline
    depth), each with its useful TFLOP/s (pack B + contraction) and its error
    against FP64."""
    import torch

    import smat
    from smat import workloads
    dev = torch.device("cuda", 0)
    A = workloads.stencil64()
    N = FORMS_WORKLOAD["N"]
    forms = {"f16": smat.FORM_F16, "bf16": smat.FORM_BF16, "fp8": smat.FORM_FP8, "split_bf16": smat.FORM_SPLIT_BF16}
    t0 = time.time()
    M = smat.Bcsr(A, forms=tuple(forms.values()))
    log(f"[bench] stencil BCSR built in {time.time() - t0:.1f}s: {M.info}")
    Bf = np.random.default_rng(7).standard_normal((A.cols, N)).astype(np.float32)
    B = torch.from_numpy(Bf).to(dev)
    Cd = torch.empty((A.rows, N), dtype=torch.float32, device=dev)
    import scipy.sparse as sps
    ref = sps.csr_matrix((A.values.astype(np.float64), A.col_idx, A.row_ptr), shape=(A.rows, A.cols)) @ \
        Bf.astype(np.float64)
    nrm = np.linalg.norm(ref)
    stream = torch.cuda.Stream(device=dev)
    sp = stream.cuda_stream
    useful = 2.0 * A.nnz * N

    def measure(Mh, f):
        ws_bytes = Mh.workspace_size(f, smat.F32, N)
        ws = torch.empty(ws_bytes, dtype=torch.uint8, device=dev)

        def step():
            Mh.spmm_raw(f, B, smat.F32, smat.ROW_MAJOR, N, Cd, smat.F32, N, N, ws, ws_bytes, sp)

        step()
        torch.cuda.synchronize(dev)
        Mh.check_device_error()
        err = float(np.linalg.norm(Cd.cpu().numpy().astype(np.float64) - ref) / nrm)
        for _ in range(max(args.warmup, 3)):
            step()
        torch.cuda.synchronize(dev)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(args.steps):
            step()
        e1.record(stream)
        torch.cuda.synchronize(dev)
        Mh.check_device_error()
        return e0.elapsed_time(e1) / args.steps, err

    best = {}   # form -> (TFLOP/s, shape, error, nnzb) of its fastest measured shape
    peak, peak_kind = peaks()

    def emit(name, shape, ms, err, info):
        v = useful / (ms * 1e-3) / 1e12
        if name not in best or v > best[name][0]:
            best[name] = (v, shape, err, info["nnzb"], info["rows_padded"])
        print(json.dumps({"metric": METRIC, "form": name, "shape": shape, "value": useful / (ms * 1e-3) / 1e12,
                          "unit": "TFLOP/s", "ms_per_step": ms, "rel_err_vs_fp64": err, "steps": args.steps,
                          "warmup": args.warmup, "higher_is_better": True, "data": "synthetic",
                          "config": dict(FORMS_WORKLOAD, nnz=A.nnz, nnzb=info["nnzb"], fill=info["fill"],
                                         panel_rows=info["panel_rows"], n_tile_cols=info["n_tile_cols"],
                                         pipeline_depth=info["pipeline_depth"])}), flush=True)

    for name, f in forms.items():
        ms, err = measure(M, f)
        emit(name, "default", ms, err, M.info)
    M.close()
    if not args.no_tune:
        for name, f in forms.items():
            t0 = time.time()
            r = smat.autotune(A, form=f, N=N)
            log(f"[bench] {name}: autotune {r} in {time.time() - t0:.0f}s")
            Mt = smat.Bcsr(A, forms=(f,), panel_rows=r["panel_rows"], split_frac=r["split_frac"],
                           n_tile_cols=r["n_tile_cols"], pipeline_depth=r["pipeline_depth"])
            ms, err = measure(Mt, f)
            emit(name, "autotuned", ms, err, Mt.info)
            Mt.close()
    # the metric's comparison: the fastest form within its error bound
    # against plain FP16, each form at its fastest measured shape
    per = {}
    for name, (v, shape, err, nnzb, rows_p) in best.items():
        fb = nnzb * (FORM_A_BYTES[name] + 4) + (rows_p // 16 + 1) * 4 + A.cols * N * 4 + A.rows * N * 4
        per[name] = {"value": v, "shape": shape, "rel_err_vs_fp64": err, "bound": FORM_BOUNDS[name],
                     "within_bound": err <= FORM_BOUNDS[name],
                     "roofline_frac_step": fb * v * 1e12 / useful / 1e9 / peak}
    ok = {n: d for n, d in per.items() if d["within_bound"]}
    chosen = max(ok, key=lambda n: ok[n]["value"]) if ok else None
    print(json.dumps({"metric": METRIC, "form": "chosen", "chosen": chosen,
                      "value": per[chosen]["value"] if chosen else None, "unit": "TFLOP/s",
                      "plain_f16_value": per["f16"]["value"] if "f16" in per else None,
                      "chosen_vs_plain_f16": (per[chosen]["value"] / per["f16"]["value"])
                      if chosen and "f16" in per else None,
                      "per_form": per, "higher_is_better": True, "data": "synthetic",
                      "config": dict(FORMS_WORKLOAD, nnz=A.nnz),
                      "note": f"roofline_frac_step: the form's BCSR-minimum bytes (FP32 B read once, FP32 C) over "
                              f"its step time, of {peak_kind} HBM"}), flush=True)


def _cusparse_blocked_ell(A, perm, Bh, N, dev, steps, warmup):
    """cuSPARSE Blocked-ELL SpMM (cusparseSpMM, CUSPARSE_SPMM_BLOCKED_ELL_ALG1)
    on the reordered matrix's 16x16 blocks, every block row padded to the
    widest one, through ctypes; returns (ms, C in the reordered row order,
    ELL bytes, stored blocks) or raises with the reason."""
    import ctypes
    import glob

    import torch

    import smat
    cs = None
    for c in sorted(glob.glob("/usr/local/cuda/lib64/libcusparse.so*")) + ["libcusparse.so"]:
        try:
            cs = ctypes.CDLL(c)
            break
        except OSError:
            continue
    if cs is None:
        raise RuntimeError("libcusparse not found")
    M = smat.Bcsr(A, row_perm=perm)
    rp, ci, vals, _ = M.export()
    nbr = len(rp) - 1
    M.close()
    bpr = np.diff(rp)
    width = int(bpr.max())
    rows, cols = nbr * 16, int(A.cols + 15) // 16 * 16
    # block (i, j) of the padded grid: the j-th block of block row i
    br = np.repeat(np.arange(nbr), bpr)
    j = np.arange(rp[-1]) - np.repeat(rp[:-1], bpr)
    col_ind = np.full((nbr, width), -1, np.int32)
    col_ind[br, j] = ci // 16
    V = torch.zeros((nbr, width, 16, 16), dtype=torch.float16, device=dev)
    V[torch.from_numpy(br).to(dev), torch.from_numpy(j).to(dev)] = torch.from_numpy(vals).to(dev)
    ell_val = V.permute(0, 2, 1, 3).contiguous()            # rows x (width * 16), row-major
    del V
    d_ind = torch.from_numpy(col_ind).to(dev)
    Bd = torch.zeros((cols, N), dtype=torch.float16, device=dev)
    Bd[: A.cols] = torch.from_numpy(Bh).to(dev)
    Bc = Bd.t().contiguous()                                 # column-major K x N (ld = K)
    Cc = torch.zeros((N, rows), dtype=torch.float32, device=dev)  # column-major M x N (ld = M)
    vp = ctypes.c_void_p
    i64 = ctypes.c_int64
    cs.cusparseCreate.argtypes = [ctypes.POINTER(vp)]
    cs.cusparseDestroy.argtypes = [vp]
    cs.cusparseCreateBlockedEll.argtypes = [ctypes.POINTER(vp), i64, i64, i64, i64, vp, vp, ctypes.c_int,
                                             ctypes.c_int, ctypes.c_int]
    cs.cusparseCreateDnMat.argtypes = [ctypes.POINTER(vp), i64, i64, i64, vp, ctypes.c_int, ctypes.c_int]
    cs.cusparseDestroySpMat.argtypes = [vp]
    cs.cusparseDestroyDnMat.argtypes = [vp]
    cs.cusparseSpMM_bufferSize.argtypes = [vp, ctypes.c_int, ctypes.c_int, vp, vp, vp, vp, vp, ctypes.c_int,
                                            ctypes.c_int, ctypes.POINTER(ctypes.c_size_t)]
    cs.cusparseSpMM.argtypes = [vp, ctypes.c_int, ctypes.c_int, vp, vp, vp, vp, vp, ctypes.c_int, ctypes.c_int, vp]
    R16F, R32F, IDX32, BASE0, ORDER_COL, ALG = 2, 0, 2, 0, 1, 13   # cuda_runtime / cusparse.h enum values
    h = vp()
    st = cs.cusparseCreate(ctypes.byref(h))
    if st:
        raise RuntimeError(f"cusparseCreate: status {st}")
    mA, mB, mC = vp(), vp(), vp()
    try:
        st = cs.cusparseCreateBlockedEll(ctypes.byref(mA), rows, cols, 16, width * 16, vp(d_ind.data_ptr()),
                                         vp(ell_val.data_ptr()), IDX32, BASE0, R16F)
        st = st or cs.cusparseCreateDnMat(ctypes.byref(mB), cols, N, cols, vp(Bc.data_ptr()), R16F, ORDER_COL)
        st = st or cs.cusparseCreateDnMat(ctypes.byref(mC), rows, N, rows, vp(Cc.data_ptr()), R32F, ORDER_COL)
        if st:
            raise RuntimeError(f"descriptor creation: status {st}")
        alpha, beta = ctypes.c_float(1.0), ctypes.c_float(0.0)
        pa, pb = ctypes.cast(ctypes.byref(alpha), vp), ctypes.cast(ctypes.byref(beta), vp)
        nbytes = ctypes.c_size_t(0)
        st = cs.cusparseSpMM_bufferSize(h, 0, 0, pa, mA, mB, pb, mC, R32F, ALG, ctypes.byref(nbytes))
        if st:
            raise RuntimeError(f"cusparseSpMM_bufferSize: status {st}")
        buf = torch.empty(max(int(nbytes.value), 16), dtype=torch.uint8, device=dev)

        def call():
            r = cs.cusparseSpMM(h, 0, 0, pa, mA, mB, pb, mC, R32F, ALG, vp(buf.data_ptr()))
            if r:
                raise RuntimeError(f"cusparseSpMM: status {r}")

        call()
        torch.cuda.synchronize(dev)
        for _ in range(max(warmup, 3)):
            call()
        torch.cuda.synchronize(dev)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        for _ in range(steps):
            call()
        e1.record()
        torch.cuda.synchronize(dev)
        ms = e0.elapsed_time(e1) / steps
        out = Cc.t()[: A.rows].double().cpu().numpy()
    finally:
        if mA:
            cs.cusparseDestroySpMat(mA)
        if mB:
            cs.cusparseDestroyDnMat(mB)
        if mC:
            cs.cusparseDestroyDnMat(mC)
        cs.cusparseDestroy(h)
    return ms, out, ell_val.numel() * 2 + d_ind.numel() * 4, nbr * width


def run_libraries(args):
    """Library comparison on the R-MAT workload: cuSPARSE CSR SpMM (through
    torch.sparse.mm) on the same A and B as the headline line, one JSON line
    per library configuration with its useful TFLOP/s and error vs FP64. A
    reported comparison, not a target and not on the product path."""
    import torch

    dev = torch.device("cuda", 0)
    A, _ = build_matrix()
    N = WORKLOAD["N"]
    Bh = np.random.default_rng(2).uniform(-1, 1, (A.cols, N)).astype(np.float16)
    import scipy.sparse as sps
    ref = sps.csr_matrix((A.values.astype(np.float64), A.col_idx, A.row_ptr), shape=(A.rows, A.cols)) @ \
        Bh.astype(np.float64)
    nrm = np.linalg.norm(ref)
    useful = 2.0 * A.nnz * N
    crow = torch.from_numpy(A.row_ptr.astype(np.int32)).to(dev)
    col = torch.from_numpy(A.col_idx.astype(np.int32)).to(dev)
    for name, dt in (("cuSPARSE CSR SpMM, FP32 values and B (torch.sparse.mm)", torch.float32),
                     ("cuSPARSE CSR SpMM, FP16 values and B (torch.sparse.mm)", torch.float16)):
        try:
            vals = torch.from_numpy(A.values.astype(np.float32)).to(dev, dt)
            S = torch.sparse_csr_tensor(crow, col, vals, size=(A.rows, A.cols), device=dev)
            B = torch.from_numpy(Bh).to(dev, dt)
            out = torch.sparse.mm(S, B)
            torch.cuda.synchronize(dev)
        except Exception as e:  # a dtype the installed torch does not route to cuSPARSE
            print(json.dumps({"metric": METRIC, "library": name, "unavailable": str(e).splitlines()[0][:200]}),
                  flush=True)
            continue
        err = float(np.linalg.norm(out.double().cpu().numpy() - ref) / nrm)
        for _ in range(max(args.warmup, 3)):
            torch.sparse.mm(S, B)
        torch.cuda.synchronize(dev)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        for _ in range(args.steps):
            torch.sparse.mm(S, B)
        e1.record()
        torch.cuda.synchronize(dev)
        ms = e0.elapsed_time(e1) / args.steps
        print(json.dumps({"metric": METRIC, "library": name, "value": useful / (ms * 1e-3) / 1e12,
                          "unit": "TFLOP/s", "ms_per_step": ms, "rel_err_vs_fp64": err, "steps": args.steps,
                          "warmup": args.warmup, "higher_is_better": True, "data": "synthetic",
                          "config": {k: WORKLOAD[k] for k in ("workload", "generator", "N", "B", "C")} |
                          {"nnz": A.nnz, "A": "CSR in the original row order (no reorder needed)",
                           "step": "one torch.sparse.mm call"}}),
              flush=True)
        del S, B, out
    # Blocked-ELL, the reference's other cuSPARSE comparison (cuda_utilities.cpp:1497-1654)
    name = "cuSPARSE Blocked-ELL SpMM, 16x16 blocks of the reordered matrix, FP16 values and B, FP32 C"
    try:
        _, perm = build_matrix()
        ms, outp, ell_bytes, stored = _cusparse_blocked_ell(A, perm, Bh, N, dev, args.steps, args.warmup)
        err = float(np.linalg.norm(outp - ref[perm]) / nrm)
        print(json.dumps({"metric": METRIC, "library": name, "value": useful / (ms * 1e-3) / 1e12,
                          "unit": "TFLOP/s", "ms_per_step": ms, "rel_err_vs_fp64": err, "steps": args.steps,
                          "warmup": args.warmup, "higher_is_better": True, "data": "synthetic",
                          "config": {k: WORKLOAD[k] for k in ("workload", "generator", "N", "B", "C")} |
                          {"nnz": A.nnz, "A": "Blocked-ELL, every block row padded to the widest "
                           f"({stored} stored blocks, {ell_bytes / 1e9:.2f} GB)",
                           "step": "one cusparseSpMM call (CUSPARSE_SPMM_BLOCKED_ELL_ALG1)"}}), flush=True)
    except Exception as e:  # the library or the format unavailable on this machine
        print(json.dumps({"metric": METRIC, "library": name, "unavailable": str(e).splitlines()[0][:200]}),
              flush=True)


PRUNED24_WORKLOAD = {
    "workload": "pruned24_randomblock65536_N128",
    "generator": "65536 x 65536, random 16x16 blocks at 2 % block density (60-90 % fill), then every block "
                 "rewritten to an exact 2:4 pattern (2 nonzeros in every aligned group of 4 columns of every "
                 "row, values N(0,1)): a 2:4-pruned block-sparse matrix; B 65536x128 FP16 U[-1,1]; FP32 C",
    "N": 128,
}


def run_pruned24(args):
    """The structured-sparse path where every block is exactly 2:4: one JSON
    line for the dense path and one per 2:4 routing threshold (use_24 = the
    fewest exact-2:4 blocks a unit of 8 block rows x 32 columns must hold)."""
    import torch

    import smat
    from smat import generators as G
    dev = torch.device("cuda", 0)
    A = G.force_24(G.random_block(65536, 0.02, 0.6, 0.9, seed=3), 1.0, seed=4)
    N = PRUNED24_WORKLOAD["N"]
    Bh = np.random.default_rng(1).uniform(-1, 1, (A.cols, N)).astype(np.float16)
    import scipy.sparse as sps
    ref = sps.csr_matrix((A.values.astype(np.float64), A.col_idx, A.row_ptr), shape=(A.rows, A.cols)) @ \
        Bh.astype(np.float64)
    B = torch.from_numpy(Bh).to(dev)
    useful = 2.0 * A.nnz * N
    for unit_min in (0, 1, 8):
        M = smat.Bcsr(A, use_24=unit_min)
        C = M.spmm(B)
        torch.cuda.synchronize(dev)
        M.check_device_error()
        err = float(np.linalg.norm(C.double().cpu().numpy() - ref) / np.linalg.norm(ref))
        ws = torch.empty(M.workspace_size(smat.FORM_F16, smat.F16, N), dtype=torch.uint8, device=dev)
        for _ in range(max(args.warmup, 3)):
            M.spmm(B, out=C, workspace=ws)
        torch.cuda.synchronize(dev)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        for _ in range(args.steps):
            M.spmm(B, out=C, workspace=ws)
        e1.record()
        torch.cuda.synchronize(dev)
        M.check_device_error()
        ms = e0.elapsed_time(e1) / args.steps
        inf = M.info
        n24 = inf["n_blocks_24"]
        print(json.dumps({"metric": METRIC, "value": useful / (ms * 1e-3) / 1e12, "unit": "TFLOP/s",
                          "ms_per_step": ms, "steps": args.steps, "warmup": args.warmup, "higher_is_better": True,
                          "data": "synthetic", "dtype": "f16", "rel_err_vs_fp64": err,
                          "config": {k: PRUNED24_WORKLOAD[k] for k in ("workload", "generator", "N")} |
                          {"nnz": A.nnz, "nnzb": inf["nnzb"], "use_24": unit_min, "n_blocks_24": n24,
                           "a_bytes": (inf["nnzb"] - n24) * 512 + n24 * 288,
                           "step": "pack B + dense SpMM" + (" + 2:4 B windows + tcgen05.mma.sp SpMM" if n24 else "")
                           + ", eager calls"}}), flush=True)
        M.close()
        del C, ws


BATCH_WORKLOAD = {
    "workload": "batched512_uneven",
    "generator": "512 matrices, rows log-uniform in [1024, 32768]; 1/3 band (half-bandwidth 8-256), 1/3 R-MAT "
                 "(average degree 8-64), 1/3 random 16x16 blocks (1-5 % block density, 40-90 % fill); "
                 "N in {32, 64, 128}; FP16 or BF16 A and B; FP32 C",
    "grouped": "smat_group_run (grouped B packing + one persistent SpMM launch) replayed from a CUDA graph",
    "sequential": "512 smat_spmm calls (pack + SpMM each) on one stream",
}


def run_batched(args):
    """Many uneven SpMMs: one grouped launch (CUDA graph) against sequential single calls."""
    import torch

    import smat
    from smat import workloads
    dev = torch.device("cuda", 0)
    count = args.batch_count
    t0 = time.time()
    probs = []
    useful = 0.0
    for A, N, fk in workloads.batched512(count):
        form = smat.FORM_F16 if fk == 0 else smat.FORM_BF16
        tdt = torch.float16 if form == smat.FORM_F16 else torch.bfloat16
        M = smat.Bcsr(A, forms=(form,))
        B = torch.randn((A.cols, N), device=dev).to(tdt)
        Cg = torch.empty((A.rows, N), dtype=torch.float32, device=dev)
        Cs = torch.empty_like(Cg)
        ws = torch.empty(M.workspace_size(form, smat.F16 if form == smat.FORM_F16 else smat.BF16, N),
                         dtype=torch.uint8, device=dev)
        probs.append((M, form, B, Cg, Cs, ws, N))
        useful += 2.0 * A.nnz * N
    log(f"[bench] {count} matrices built in {time.time() - t0:.1f}s, useful {useful / 1e9:.2f} GFLOP")
    stream = torch.cuda.Stream(device=dev)
    sp = stream.cuda_stream

    def sequential():
        for M, form, B, Cg, Cs, ws, N in probs:
            M.spmm(B, form=form, out=Cs, workspace=ws, stream=sp)

    g = smat.Group([(M, form, B, Cg) for M, form, B, Cg, Cs, ws, N in probs])
    g.run(sp)
    stream.synchronize()
    graph = torch.cuda.CUDAGraph()
    with torch.cuda.graph(graph, stream=stream):
        g.run(sp)

    def timed(fn, reps):
        for _ in range(max(args.warmup, 3)):
            fn()
        torch.cuda.synchronize(dev)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(reps):
            fn()
        e1.record(stream)
        torch.cuda.synchronize(dev)
        return e0.elapsed_time(e1) / reps

    with torch.cuda.stream(stream):
        ms_seq = timed(sequential, max(2, args.steps // 5))
        ms_grp = timed(graph.replay, args.steps)
    g.check_device_error()
    diff = max(float((Cg - Cs).abs().max() / Cs.abs().max().clamp_min(1e-30)) for M, f, B, Cg, Cs, ws, N in probs)
    print(json.dumps({"metric": METRIC, "workload": BATCH_WORKLOAD["workload"],
                      "value": useful / (ms_grp * 1e-3) / 1e12, "unit": "TFLOP/s", "ms_per_step": ms_grp,
                      "sequential": {"value": useful / (ms_seq * 1e-3) / 1e12, "ms_per_step": ms_seq},
                      "speedup_vs_sequential": ms_seq / ms_grp, "max_rel_diff_grouped_vs_sequential": diff,
                      "steps": args.steps, "warmup": args.warmup, "higher_is_better": True, "data": "synthetic",
                      "config": dict(BATCH_WORKLOAD, count=count, useful_gflop=useful / 1e9)}), flush=True)
    g.close()


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=50)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="smat", choices=["smat", "reference"])
    ap.add_argument("--workload", default="rmat16",
                    choices=["rmat16", "stencil64_forms", "batched512", "rmat16_libraries", "rmat16_reorder",
                             "pruned24", "rmat16_tiles"],
                    help="rmat16: the headline SpMM line; stencil64_forms: one line per precision form; "
                         "batched512: grouped vs sequential SpMMs; rmat16_libraries: cuSPARSE on the "
                         "headline inputs, for comparison; rmat16_reorder: the reorder step alone "
                         "(with --impl reference: the reference's own reorder); rmat16_tiles: the merged "
                         "4 x 4-block tiles built on the GPU and the _tiled launchers on them")
    ap.add_argument("--batch-count", type=int, default=512)
    ap.add_argument("--no-sp24", action="store_true", help="skip the structured-sparse (2:4) path's line")
    ap.add_argument("--no-forms", action="store_true", help="rmat16: skip the other precision forms")
    ap.add_argument("--no-tune", action="store_true", help="stencil forms: skip the autotuned lines")
    ap.add_argument("--reorder-gpu", action="store_true", help="rmat16_reorder: candidate distances on the GPU")
    args = ap.parse_args()
    if args.workload == "rmat16_reorder":
        run_reorder(args)
    elif args.impl == "reference":
        run_reference(args)
    elif args.workload == "stencil64_forms":
        run_forms(args)
    elif args.workload == "batched512":
        run_batched(args)
    elif args.workload == "rmat16_libraries":
        run_libraries(args)
    elif args.workload == "pruned24":
        run_pruned24(args)
    elif args.workload == "rmat16_tiles":
        run_tiles(args)
    else:
        run_smat(args)


if __name__ == "__main__":
    main()
