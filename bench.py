#!/usr/bin/env python3
"""Benchmark: masked SpGEMM GFLOP/s on the k-truss sweep of an R-MAT graph.

Workload (one step): the k-truss sweep k = 3, 4, ... up to the largest k with
a non-empty truss, on a seeded R-MAT graph (scale 18, edge factor 16,
a/b/c/d = 0.57/0.19/0.19/0.05, symmetrised, loops and duplicates removed,
int32 CSR, 262,144 vertices, 7.6M stored entries). Each k runs the
reference's k_truss (src/main.cpp:90-146: Tmp<C> = C*C masked by C, prune
below k-2, repeat until nnz is unchanged) through the C ABI, the support
product by triangle listing by default (GA_TRI: each triangle found once
over a degree orientation and counted on its three edges; --algo
msa|mca|heap|dot|hybrid runs one of the other forms);
k starts from the (k-1)-truss, which contains it (same edge sets as starting
from A). value = 2 * (Gustavson products of every support product, the work
of the reference's C<M> = A*B whatever form computes it) / time, inputs
resident in HBM, L2 flushed (256 MiB write) between steps: a
reference-equivalent rate (unit "reference-equivalent GFLOP/s"), since the
triangle-listing form reaches the same supports with far fewer operations.

e2e: the same sweep through the public API from pinned host buffers: upload
A, run the sweep, download every k-truss (row starts and columns).

parity: every k-truss the e2e sweep downloaded (iteration count, entries,
edge-set digest) against the oracle's record of the same sweep
(tests/golden/rmat18_sweep.json), the k = 3 truss against the oracle run
live, TC and BC of the other configurations against the oracle.

cpu_baseline / --impl reference: the oracle port of the reference's k_truss
(oracle/oracle.c, OpenMP over all host cores) on a bounded sample of the same
workload - the k = 3 stage from A - reported in the same unit. The reference
arm loads nothing of the product: its graph comes from the oracle's copy of
the generator (oracle/gen.c).

The default line also carries the other configurations: the triangle count
of an Erdos-Renyi graph (n = 1,000), batched BC on R-MAT scale 20 (64 and 256
sources), the batched TC + 4-truss of 4,096 k-NN graphs against per-graph
launches, and the request server against the plain sequential form.

Multi-GPU: the path does not shard; --gpus N under torchrun runs N
independent replicas (one per rank) and reports their aggregate.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

METRIC = "masked SpGEMM GFLOP/s & HBM % of peak; batched/served req/s, p50/p99 vs plain"
UNIT = "reference-equivalent GFLOP/s"
HBM_FALLBACK_GBS = 6800.0
GOLDEN_SWEEP = os.path.join(ROOT, "tests", "golden", "rmat18_sweep.json")
# DRAM bytes per stored entry of the dominant kernels, from one ncu capture
# each (dram__bytes_read.sum + dram__bytes_write.sum of the launch divided by
# its stored entries): k_tri_support on the first support product of the
# R-MAT 18 4-truss (profiles/tri_support_rmat18.md) and k_mxm_masked<MSA> on
# the R-MAT 18 support product (profiles/mxm_msa_rmat18_support.md). Each
# launch of the sweep works on operands that fit in L2, so its DRAM traffic
# is the compulsory traffic of its operands, proportional to its entries.
DRAM_BYTES_PER_ENTRY = {"tri_support": 7.506, "mxm": 4.543}
# DRAM bytes per pruned edge of the frontier pruning kernels (k_trif_lower +
# k_trif_lower_seg): dram__bytes_read.sum + dram__bytes_write.sum summed over
# every launch of one R-MAT 18 sweep (ncu with --cache-control none, so the
# caches stay warm as in the timed step: 1,721.0 MB) over its 3,805,777
# pruned edges (profiles/trif_lower_rmat18_sweep.md).
DRAM_BYTES_PER_FRONT_EDGE = 452.2


def parse_args():
    ap = argparse.ArgumentParser(description=__doc__.split("\n\n")[0])
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["gb300", "reference"], default="gb300")
    ap.add_argument("--scale", type=int, default=18)
    ap.add_argument("--edge-factor", type=int, default=16)
    ap.add_argument("--seed", type=int, default=42)
    ap.add_argument("--algo", default=None, choices=["msa", "mca", "heap", "dot", "hybrid", "tri", "auto"],
                    help="k-truss variant (default: tri for the sweep, msa for --case, auto for the batch "
                         "workload)")
    ap.add_argument("--kmin", type=int, default=3)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--hybrid-ratio", type=int, default=None,
                    help="hybrid variant: work ratio above which a row goes to the inner-product form")
    ap.add_argument("--tune", action="store_true",
                    help="k-truss sweep: use the bin thresholds tuned on the first support product "
                         "(slower over the whole sweep, whose later graphs are small)")
    ap.add_argument("--no-other-configs", action="store_true",
                    help="skip the TC (Erdos-Renyi n=1000) and BC (R-MAT 20) measurements")
    ap.add_argument("--cpu-reps", type=int, default=2)
    ap.add_argument("--case", choices=["support", "tc", "bc", "ktruss", "sweep", "batch"], default=None,
                    help="profiling case instead of the benchmark, --reps times: support product, TC, BC, "
                         "4-truss from A, the k-truss sweep from A, or batched TC + 4-truss of --graphs k-NN "
                         "graphs")
    ap.add_argument("--reps", type=int, default=2)
    ap.add_argument("--sources", type=int, default=64)
    ap.add_argument("--bc-backward", type=int, default=None, choices=[0, 1, 2],
                    help="BC case: how the backward sweep reads W rows (GA_OPT_BC_BACKWARD: 0 gathers, "
                         "1 bulk copies, 2 one neighbour at a time)")
    ap.add_argument("--ingest-scale", type=int, default=20, help="ingest workload: R-MAT scale of the file")
    ap.add_argument("--workload", choices=["ktruss-sweep", "batch", "serve", "ingest"], default="ktruss-sweep",
                    help="ktruss-sweep: the R-MAT k-truss sweep; batch: TC + 4-truss of many k-NN graphs; "
                         "serve: a stream of TC / k-truss / BC requests on a pool of resident graphs")
    ap.add_argument("--requests", type=int, default=300, help="serve workload: requests per run")
    ap.add_argument("--workers", type=int, default=4, help="serve workload: server worker threads")
    ap.add_argument("--serve-algo", default="auto", choices=["msa", "mca", "heap", "dot", "auto"],
                    help="serve workload: variant of single TC / k-truss requests (both forms)")
    ap.add_argument("--rmat-scales", default="10,12,14,16,18,20,22", help="serve workload: R-MAT pool scales")
    ap.add_argument("--knn-sizes", default="1000,10000,100000,1000000", help="serve workload: k-NN pool sizes")
    ap.add_argument("--rates", default="0.5,1,2,4",
                    help="serve workload: Poisson rates as multiples of the plain form's throughput")
    ap.add_argument("--graphs", type=int, default=4096, help="batch workload: number of graphs")
    ap.add_argument("--plain-graphs", type=int, default=0,
                    help="batch workload: graphs timed in the per-graph arm (0 = all)")
    ap.add_argument("--tc-algo", default=None, choices=["msa", "mca", "heap", "dot", "tri", "auto"],
                    help="TC variant (default: msa; auto for the batch workload)")
    ap.add_argument("--batch-algo", default="auto", choices=["msa", "mca", "heap", "dot", "tri", "auto"],
                    help="batched record: k-truss variant of the batched calls")
    ap.add_argument("--batch-tc-algo", default="auto", choices=["msa", "mca", "heap", "dot", "tri", "auto"],
                    help="batched record: TC variant of the batched calls")
    ap.add_argument("--serve-requests", type=int, default=300,
                    help="default line: requests of the light-mix serving record")
    ap.add_argument("--serve-full-requests", type=int, default=90,
                    help="default line: requests of the full-pool serving record (0: skip it)")
    ap.add_argument("--host-loops", action="store_true",
                    help="run the k-truss loop from the host (kernels launched one by one, e.g. for ncu)")
    args = ap.parse_args()
    auto = args.workload == "batch" or args.case == "batch"
    if args.algo is None:
        args.algo = "auto" if auto else ("tri" if args.workload == "ktruss-sweep" and not args.case else "msa")
    if args.tc_algo is None:
        args.tc_algo = "auto" if auto else "msa"
    return args


# ---------------------------------------------------------------- plumbing
class Dist:
    def __init__(self):
        self.world = int(os.environ.get("WORLD_SIZE", "1"))
        self.rank = int(os.environ.get("RANK", "0"))
        self.local_rank = int(os.environ.get("LOCAL_RANK", "0"))
        self.pg = None
        if self.world > 1:
            import torch.distributed as td
            os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
            td.init_process_group("gloo", rank=self.rank, world_size=self.world)
            self.pg = td

    def barrier(self):
        if self.pg:
            self.pg.barrier()

    def max(self, x: float) -> float:
        if not self.pg:
            return x
        import torch
        t = torch.tensor([x], dtype=torch.float64)
        self.pg.all_reduce(t, op=self.pg.ReduceOp.MAX)
        return float(t.item())

    def sum(self, x: float) -> float:
        if not self.pg:
            return x
        import torch
        t = torch.tensor([x], dtype=torch.float64)
        self.pg.all_reduce(t, op=self.pg.ReduceOp.SUM)
        return float(t.item())

    def close(self):
        if self.pg:
            self.pg.destroy_process_group()


class ClockSampler:
    """nvidia-smi clock / throttle sampling (200 ms) during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.proc = None
        self.path = None

    def start(self):
        try:
            fd, self.path = tempfile.mkstemp(suffix=".csv")
            os.close(fd)
            self.out = open(self.path, "w")
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=self.out, stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None

    def stop(self) -> dict:
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        time.sleep(0.25)
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        self.out.close()
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        with open(self.path) as f:
            for line in f:
                parts = [x.strip() for x in line.split(",")]
                if len(parts) < 9:
                    continue
                try:
                    sm.append(float(parts[1]))
                    smax.append(float(parts[2]))
                except ValueError:
                    continue
                for nm, val in zip(names, parts[5:9]):
                    if val.lower() == "active":
                        reasons.add(nm)
        os.unlink(self.path)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def measured_peak_hbm():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            v = json.load(f).get("hbm_gbs")
        if v:
            return float(v), "measured"
    except Exception:
        pass
    return HBM_FALLBACK_GBS, "fallback"


def run_case(args):
    """Small profiling cases, --reps times each (used for ncu captures):
    `support` = the sweep's first support product C<A> = A*A; `tc` =
    triangle count with the dot-product kernel; `bc` = batched BC over
    --sources seeded sources; `ktruss` = 4-truss from A; `sweep` = the
    k-truss sweep k = --kmin ... from A, with the library's kernel launches
    per sweep (all on the bench's R-MAT graph); `batch` = batched TC +
    4-truss of --graphs k-NN graphs."""
    import graphalgo_gb300 as ga
    from graphalgo_gb300 import build as gbuild
    gbuild.build()
    ctx = ga.Context(0)
    ctx.set_option(ga.OPT_DEVICE_LOOPS, 0 if args.host_loops else 1)
    if args.hybrid_ratio is not None:
        ctx.set_option(ga.OPT_HYBRID_RATIO, args.hybrid_ratio)
    if args.bc_backward is not None:
        ctx.set_option(ga.OPT_BC_BACKWARD, args.bc_backward)
    if args.case == "batch":
        n, dim = knn_batch_sizes(args.graphs, args.seed)
        U, voff = ga.gen_knn_batch(ctx, n, dim, k=30, seed=args.seed)
        for _ in range(args.reps):
            ctx.work_counters(reset=True)
            ctx.timer_start()
            tcs = ga.batch_tc(args.tc_algo, U, voff)
            C, iters = ga.batch_ktruss(args.algo, U, voff, 4)
            ms = ctx.timer_stop()
            print(json.dumps({"batch_ms": ms, "graphs": args.graphs, "triangles": int(tcs.sum()),
                              "truss_entries": C.nnz, "max_iters": int(iters.max()),
                              "products": ctx.work_counters()["products"]}), flush=True)
            C.free()
        ctx.close()
        return
    m, rst, col = ga.gen_rmat(args.scale, args.edge_factor, 0.57, 0.19, 0.19, args.seed)
    A = ga.Csr.upload(ctx, m, m, rst, col, np.ones(len(col), np.int32))
    A.set_symmetric(1)  # symmetrised by construction
    rng = np.random.default_rng(args.seed)
    src = rng.choice(m, min(args.sources, m), replace=False).astype(np.int32)
    for _ in range(args.reps):
        ctx.work_counters(reset=True)
        ctx.timer_start()
        if args.case == "support":
            C = ga.mxm_masked(args.algo, A, A, A)
            ms = ctx.timer_stop()
            C.free()
            wc = ctx.work_counters()
            rec = {"support_ms": ms, "products": wc["products"], "mask_entries": wc["mask_entries"],
                   "gflops": 2.0 * wc["products"] / ms / 1e6}
        elif args.case == "tc":
            total, _ = ga.tc("dot", A, per_row=False)
            ms = ctx.timer_stop()
            ctx.timer_start()
            total_tri, _ = ga.tc("tri", A, per_row=False)
            ms_tri = ctx.timer_stop()
            rec = {"tc_ms": ms, "tc_tri_ms": ms_tri, "triangles": total, "triangles_tri": total_tri}
        elif args.case == "ktruss":
            C, it = ga.ktruss(args.algo, A, 4)
            ms = ctx.timer_stop()
            rec = {"ktruss_ms": ms, "iters": it, "nnz": C.nnz, "products": ctx.work_counters()["products"]}
            C.free()
        elif args.case == "sweep":
            l0 = ga.kernel_launches()
            shape = sweep(ga, ctx, A, args.algo, args.kmin)
            ms = ctx.timer_stop()
            rec = {"sweep_ms": ms, "stages": len(shape), "iterations": int(sum(s[1] for s in shape)),
                   "launches": ga.kernel_launches() - l0, "products": ctx.work_counters()["products"]}
        else:
            ga.bc(A, src)
            ms = ctx.timer_stop()
            rec = {"bc_ms": ms, "sources": len(src), "gteps": len(src) * len(col) / 2 / ms / 1e6}
        print(json.dumps(rec), flush=True)
    ctx.close()


def load_sweep_golden(args):
    """The oracle's record of the sweep (tests/golden/rmat18_sweep.json) when
    the arguments name the same graph, else None."""
    try:
        with open(GOLDEN_SWEEP) as f:
            rec = json.load(f)
    except OSError:
        return None
    g = rec["graph"]
    if (g["scale"], g["edge_factor"], g["seed"]) != (args.scale, args.edge_factor, args.seed) or args.kmin != 3:
        return None
    return rec


def edge_digest(rst: np.ndarray, col: np.ndarray) -> str:
    """BLAKE2b-128 of the row starts then the columns (little-endian int32),
    as the golden record holds it."""
    import hashlib
    h = hashlib.blake2b(digest_size=16)
    h.update(np.ascontiguousarray(rst, "<i4").tobytes())
    h.update(np.ascontiguousarray(col, "<i4").tobytes())
    return h.hexdigest()


def workload_config(args, m, nnz, kmax):
    """The workload, the same dict in both arms."""
    return {"workload": f"k-truss sweep k={args.kmin}..k_max, R-MAT scale {args.scale}",
            "graph": f"R-MAT scale {args.scale}, edge factor {args.edge_factor}, a/b/c/d=0.57/0.19/0.19/0.05, "
                     f"seed {args.seed}, symmetrised, no loops/duplicates",
            "vertices": m, "stored_entries": nnz, "k_range": [args.kmin, kmax],
            "k_start": "each k starts from the (k-1)-truss",
            "l2": "flushed between steps (256 MiB write)", "parallelism": "replicas only"}


def cpu_sample(A_host, reps: int):
    """Oracle port (OpenMP, all host threads) on the k=3 stage from A."""
    import oracle
    oracle.build()
    threads = os.cpu_count() or 1
    oracle.set_num_threads(threads)
    times, prod, res = [], 0, None
    for _ in range(max(1, reps)):
        t0 = time.perf_counter()
        C, it, prod = oracle.ktruss(A_host, 3, with_products=True)
        times.append(time.perf_counter() - t0)
        res = (C, it)
    t = statistics.median(times)
    return {"value": 2.0 * prod / t / 1e9, "unit": UNIT, "cores": threads, "kind": "port",
            "sample": f"k=3 stage of the sweep from A (k_truss, {prod:.4g} Gustavson products), "
                      f"median of {len(times)} runs, {t:.3f} s each"}, res


# --------------------------------------------------------------- GPU arm
def sweep(ga, ctx, A, algo, kmin, sink=None, per_k=None):
    """k-truss sweep from A: C_k = k_truss(C_{k-1}, k) until the truss is
    empty, through ga.ktruss_sweep (with triangle listing one device-resident
    state for the whole sweep). Each C_k is freed once the next one exists,
    so a download of it (sink) overlaps with the next k."""
    out, prev = [], None
    if per_k is not None:
        ctx.work_counters(reset=True)
    for k, C, it in ga.ktruss_sweep(algo, A, kmin):
        out.append((k, it, C.nnz))
        if per_k is not None:
            per_k[k] = ctx.work_counters(reset=True)
        if sink is not None:
            sink(k, C)
        if prev is not None:
            prev.free()
        prev = C
    if prev is not None:
        prev.free()
    return out


def profile_step(ga, ctx, run, algo, counters, loops):
    """Runs one step with host-driven loops and per-kernel timing; returns the
    launch count and the roofline of the step's dominant kernel.

    Gustavson variants: achieved = algorithmic bytes of the Gustavson model
    with int32 values (s = 4): 4(m+1)*2 + nnz(A)*(4+4) + nnz(A)*8 + P*(4+4) +
    nnz(M)*4 + nnz(C)*4, P being the products the kernel processed (the
    support of a symmetric C evaluates its upper triangle and mirrors it),
    divided by the kernel's summed event time. Triangle listing (the sweep
    lists the triangles once and then prunes by frontier): the frontier
    kernel k_trif_lower, 48 bytes per pruned edge (its frontier slot, row,
    column, diagonal positions, support, both rows' bounds, the oriented
    count and rank of the far row), 34 bytes per probed row entry (column,
    record position, state and rank of the entry, about four binary-search
    steps in the other row, the found entry's record position and state) and
    16 bytes per destroyed triangle (two 4-byte support read-modify-writes),
    over its summed event time."""
    ctx.set_option(ga.OPT_DEVICE_LOOPS, 0)
    ctx.set_option(ga.OPT_PROFILE, 1)
    ctx.reset_kernel_stats()
    ctx.work_counters(reset=True)
    l0 = ga.kernel_launches()
    ctx.flush_l2()
    run()
    ctx.sync()
    launches = ga.kernel_launches() - l0
    stats = ctx.kernel_stats()
    ctr = counters()
    ctx.set_option(ga.OPT_PROFILE, 0)
    ctx.set_option(ga.OPT_DEVICE_LOOPS, loops)
    kname = {"msa": "mxm_msa", "mca": "mxm_mca", "heap": "mxm_heap_merge", "dot": "mxm_dot",
             "hybrid": "mxm_msa", "tri": "trif_lower"}[algo]
    k_launches, k_ms = stats.get(kname, (0, 0.0))
    if algo == "tri":
        bytes_model = 48 * ctr["front_edges"] + 34 * ctr["front_probes"] + 16 * ctr["front_triangles"]
        tpe = DRAM_BYTES_PER_FRONT_EDGE
        traffic_units = ctr["front_edges"]  # the capture's DRAM bytes are per pruned edge
    else:
        # products of the Gustavson kernels; list entries walked for the inner-product one
        ex = ctr["executed_dot"] if algo == "dot" else ctr["executed"]
        bytes_model = 8 * ctr["rows"] + 16 * ctr["a_entries"] + 8 * ex + 8 * ctr["mask_entries"]
        tpe = DRAM_BYTES_PER_ENTRY["mxm"]
        traffic_units = ctr["mask_entries"]
    peak, peak_kind = measured_peak_hbm()
    achieved = bytes_model / (k_ms * 1e-3) / 1e9 if k_ms > 0 else None
    traffic = (tpe * traffic_units / max(1, k_launches)) if tpe is not None else None
    return {"launches": launches, "kernel_ms": k_ms, "stats": stats, "counters": ctr,
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                         "frac": (achieved / peak) if achieved else None, "traffic": traffic,
                         "kernel": kname, "peak_kind": peak_kind,
                         "bytes_per_launch": bytes_model / max(1, k_launches),
                         "avg_launch_ms": k_ms / max(1, k_launches)}}


def bc_bytes_model(m, rst, col, src):
    """Algorithmic bytes of a batched BC call under the Gustavson model of
    the reference's algebra (betweenness_centrality.h:176-218): every source
    s walks the stored entries of its connected component once forward
    (Front<!Numsp> = A^T * Front: a 4-byte column and an 8-byte path count
    per entry) and once backward (W<S[k-1]> = A * W: the same), and per
    (vertex, source) pair reached writes its path count, reads it back,
    writes its dependency and adds it into bc (4 x 8 bytes) plus its column
    in the frontier (4 bytes)."""
    import scipy.sparse as sp
    from scipy.sparse.csgraph import connected_components
    G = sp.csr_matrix((np.ones(len(col), np.int8), col, rst), shape=(m, m))
    _, lab = connected_components(G, directed=False)
    ent = np.bincount(lab, weights=np.diff(rst), minlength=lab.max() + 1)
    ver = np.bincount(lab, minlength=lab.max() + 1)
    e = float(ent[lab[src]].sum())
    v = float(ver[lab[src]].sum())
    return 2 * 12 * e + 36 * v


def other_configs(ga, ctx, args, with_cpu: bool):
    """The other single-GPU workloads, measured beside the headline: the
    triangle count of a seeded Erdos-Renyi graph (n=1000, 9,990 edges, uint8
    values; latency, bit-exact against the oracle) and batched BC on R-MAT
    scale 20 with 64 and 256 seeded sources (FP64; GTEPS = sources * nnz / 2
    / t), the 64-source scores checked against the FP64 oracle (1e-9
    relative), which is also timed on all host cores as the CPU baseline."""
    import oracle
    out = {}
    # triangle count, Erdos-Renyi n = 1000
    m, rst, col = ga.gen_er(1000, 9990, seed=args.seed)
    A8 = ga.Csr.upload(ctx, m, m, rst, col, np.ones(len(col), np.uint8))
    ref_total, ref_rows = oracle.tc_sandia(oracle.Csr(m, m, rst, col, np.ones(len(col), np.int32)))
    rec = {}
    tot = ga.Dense.create(ctx, 1, 1, ga.INT64)
    exact = True
    for algo in ("msa", "dot", "tri"):
        got, rows = ga.tc(algo, A8 if algo != "tri" else ga.Csr.upload(ctx, m, m, rst, col))
        exact = exact and got == ref_total and bool(np.array_equal(rows, ref_rows))
        if algo == "tri":
            continue
        reps = 200
        ctx.sync()
        ctx.timer_start()
        for _ in range(reps):
            ga.tc_device(algo, A8, tot)
        rec[algo + "_us"] = 1e3 * ctx.timer_stop() / reps
    # e2e: upload (the host CSR's pattern; unit uint8 values set on the
    # device, the graph declared symmetric as generated), count, per-row
    # counts back to the host
    reps = 50
    t0 = time.perf_counter()
    for _ in range(reps):
        X = ga.Csr.upload(ctx, m, m, rst, col, dtype=ga.UINT8)
        X.set_symmetric(1)
        ga.tc("dot", X)
        X.free()
    rec["e2e_dot_us"] = 1e6 * (time.perf_counter() - t0) / reps
    Gh = oracle.Csr(m, m, rst, col, np.ones(len(col), np.int32))
    oracle.set_num_threads(os.cpu_count() or 1)
    t0 = time.perf_counter()
    for _ in range(reps):
        oracle.tc_sandia(Gh)
    rec["cpu_port_us"] = 1e6 * (time.perf_counter() - t0) / reps
    rec["cpu_port_threads"] = os.cpu_count() or 1
    out["tc_er1000"] = {"triangles": ref_total, "edges": len(col) // 2, "bit_exact": exact, **rec,
                        "note": "device time per call (CUDA events, 200 calls, graph resident); e2e includes "
                                "the pattern's upload and validation and the per-row download (wall time, 50 "
                                "calls); bit_exact: total and per-row counts of the MSA, inner-product and "
                                "triangle-listing forms against the oracle"}
    # batched BC, R-MAT scale 20
    m, rst, col = ga.gen_rmat(20, 16, 0.57, 0.19, 0.19, args.seed)
    A = ga.Csr.upload(ctx, m, m, rst, col, np.ones(len(col), np.int32))
    rng = np.random.default_rng(args.seed)
    peak, peak_kind = measured_peak_hbm()
    for ns in (64, 256):
        src = rng.choice(m, ns, replace=False).astype(np.int32)
        got = ga.bc(A, src)
        ms = []
        for _ in range(3):
            ctx.flush_l2()
            ctx.timer_start()
            ga.bc(A, src)
            ms.append(ctx.timer_stop())
        t = min(ms)
        bm = bc_bytes_model(m, rst, col, src)
        r = {"ms": t, "gteps": ns * len(col) / 2 / t / 1e6, "runs_ms": ms, "unit": "GTEPS",
             "roofline": {"bound": "hbm", "achieved": bm / (t * 1e-3) / 1e9, "peak": peak, "unit": "GB/s",
                          "frac": bm / (t * 1e-3) / 1e9 / peak, "traffic": None, "peak_kind": peak_kind,
                          "bytes_per_call": bm, "scope": "whole BC call (forward and backward sweeps)"}}
        if ns == 64 and with_cpu:
            oracle.set_num_threads(os.cpu_count() or 1)
            Ah = oracle.Csr(m, m, rst, col, np.ones(len(col), np.int32))
            t0 = time.perf_counter()
            ref = oracle.bc_batch(Ah, src)
            tc = time.perf_counter() - t0
            rel = np.abs(got - ref) / np.maximum(np.abs(ref), 1.0)
            r["parity"] = {"max_rel_err": float(rel.max()), "within_1e-9": bool(rel.max() <= 1e-9),
                           "against": "FP64 oracle (oracle.bc_batch), same sources"}
            r["cpu_baseline"] = {"value": ns * len(col) / 2 / tc / 1e9, "unit": "GTEPS",
                                 "cores": os.cpu_count() or 1, "kind": "port",
                                 "sample": f"the same call ({ns} sources, FP64) by the oracle port, {tc:.2f} s"}
        out[f"bc_rmat20_{ns}src"] = r
    # the masked product itself on the same graph (31.4M entries: operands
    # larger than L2), C<A> = A*A with int32 values, default schedule, per
    # Gustavson variant against the survey's byte model 8(m+1) + 16 nnz(A) +
    # 8 P + 4 nnz(M) + 4 nnz(C); triangle listing (which performs no
    # Gustavson products) by time only
    nnz = len(col)
    mx = {}
    for algo in ("msa", "hybrid", "mca", "tri"):
        ga.mxm_masked(algo, A, A, A).free()
        best, prods = None, 0
        for _ in range(2):
            ctx.work_counters(reset=True)
            ctx.flush_l2()
            ctx.timer_start()
            C = ga.mxm_masked(algo, A, A, A)
            t = ctx.timer_stop()
            C.free()
            prods = ctx.work_counters(reset=True)["products"]
            best = t if best is None else min(best, t)
        rec = {"ms": best, "reference_equivalent_gflops": 2.0 * prods / best / 1e6}
        if algo != "tri":
            bm = 8 * (m + 1) + 16 * nnz + 8 * prods + 4 * nnz + 4 * nnz
            rec["roofline"] = {"bound": "hbm", "achieved": bm / (best * 1e-3) / 1e9, "peak": peak, "unit": "GB/s",
                               "frac": bm / (best * 1e-3) / 1e9 / peak, "bytes_per_call": bm,
                               "peak_kind": peak_kind, "traffic": None}
        mx[algo] = rec
    out["mxm_rmat20"] = {"product": "C<A> = A*A (the k-truss support), R-MAT scale 20, int32 values",
                         "gustavson_products": prods, "variants": mx}
    return out


def run_gpu(args, dist: Dist):
    import graphalgo_gb300 as ga
    from graphalgo_gb300 import build as gbuild
    gbuild.build()
    ctx = ga.Context(dist.local_rank)
    loops = 0 if args.host_loops else 1
    ctx.set_option(ga.OPT_DEVICE_LOOPS, loops)
    if args.hybrid_ratio is not None:
        ctx.set_option(ga.OPT_HYBRID_RATIO, args.hybrid_ratio)
    golden = load_sweep_golden(args)

    m, rst, col = ga.gen_rmat(args.scale, args.edge_factor, 0.57, 0.19, 0.19, args.seed)
    nnz = len(col)
    val = np.ones(nnz, np.int32)
    A = ga.Csr.upload(ctx, m, m, rst, col, val)
    # the variant's bin thresholds and grid size, tuned on the first support product
    schedule = None
    if args.tune and args.algo in ("msa", "mca", "dot"):
        schedule = ga.autotune(ga.TUNE_KTRUSS, A, only=args.algo)
        ga.apply_schedule(ctx, schedule)

    # warm-up (also fixes k_max)
    shape = None
    for _ in range(max(1, args.warmup)):
        shape = sweep(ga, ctx, A, args.algo, args.kmin)
    kmax = shape[-1][0] - 1 if len(shape) > 1 else args.kmin

    # ------------------------------------------------------- timed region
    sampler = ClockSampler(dist.local_rank)
    ctx.work_counters(reset=True)
    dist.barrier()
    ctx.sync()
    sampler.start()
    step_ms = []
    for _ in range(args.steps):
        ctx.flush_l2()
        ctx.timer_start()
        sweep(ga, ctx, A, args.algo, args.kmin)
        step_ms.append(ctx.timer_stop())
    ctx.sync()
    clocks = sampler.stop()
    dist.barrier()
    wc = ctx.work_counters(reset=True)
    total_ms = sum(step_ms)
    flops = 2.0 * wc["products"]
    t_max = dist.max(total_ms)
    flops_all = dist.sum(flops)
    value = flops_all / (t_max * 1e-3) / 1e9

    # ----------------------------------- per-kernel profile of one step
    per_k = {}
    prof = profile_step(ga, ctx, lambda: sweep(ga, ctx, A, args.algo, args.kmin, per_k=per_k), args.algo,
                        lambda: {key: sum(v[key] for v in per_k.values()) for key in next(iter(per_k.values()))},
                        loops)
    launches_per_step = prof["launches"]
    roofline = prof["roofline"]
    roofline["kernel_share_of_step"] = prof["kernel_ms"] / (total_ms / args.steps) if total_ms else None

    # ---------------------------------------------------------- e2e
    # the sweep through the public API from pinned host buffers; every
    # k-truss it downloads is then checked against the oracle's record
    rst_h = np.ascontiguousarray(rst, np.int32)
    col_h = np.ascontiguousarray(col, np.int32)
    res_rst = np.empty((len(shape), m + 1), np.int32)
    res_col = np.empty(sum(s[2] for s in shape) + 1, np.int32)
    pinned = [rst_h, col_h, res_rst, res_col]
    for a in pinned:
        ga.host_register(a)
    e2e, got_shape = None, None
    try:
        d2h = 0

        def sink_factory():
            state = {"i": 0, "off": 0}

            def sink(k, C):
                nonlocal d2h
                z = C.nnz
                r = res_rst[state["i"]]
                c = res_col[state["off"]:state["off"] + z]
                # on the copy stream: overlaps with the next k's pruning
                ga.lib().ga_csr_download_async(ctx.handle, C.handle, r.ctypes.data_as(ga._p),
                                               c.ctypes.data_as(ga._p), None)
                d2h += (m + 1) * 4 + z * 4
                state["i"] += 1
                state["off"] += z
            return sink

        e2e_ms = []
        dist.barrier()
        # one untimed pass first (the e2e path's own warm-up), then the steps
        for step in range(-1, 1 if args.no_e2e else args.steps):
            if step == 0:
                ctx.work_counters(reset=True)
            ctx.flush_l2()
            d2h = 0
            ctx.timer_start()
            # the pattern only: an adjacency matrix's values are all 1 (the
            # reference CLI's build_adjacency_matrix), set on the device
            Ad = ga.Csr.upload(ctx, m, m, rst_h, col_h)
            Ad.set_symmetric(1)  # symmetrised by construction, as the reference CLI's graphs are
            got_shape = sweep(ga, ctx, Ad, args.algo, args.kmin, sink=sink_factory())
            Ad.free()
            ga.lib().ga_ctx_copy_sync(ctx.handle)
            t_e2e = ctx.timer_stop()
            if step >= 0:
                e2e_ms.append(t_e2e)
        wce = ctx.work_counters(reset=True)
        if not args.no_e2e:
            e2e_t = dist.max(sum(e2e_ms))
            e2e = {"value": dist.sum(2.0 * wce["products"]) / (e2e_t * 1e-3) / 1e9, "unit": UNIT,
                   "h2d_bytes_per_step": int(rst_h.nbytes + col_h.nbytes),
                   "d2h_bytes_per_step": int(d2h), "ms_per_step": e2e_t / args.steps,
                   "runs_ms": [round(x, 3) for x in e2e_ms],
                   "note": "per step: upload of A's pattern from pinned host memory (values all 1, set on the "
                           "device; validated on the device, declared symmetric with ga_csr_set_symmetric), "
                           "the sweep, every k-truss downloaded"}
        # digests of every downloaded k-truss
        digests, off = [], 0
        for i, (k, it, z) in enumerate(got_shape):
            digests.append([k, it, z, edge_digest(res_rst[i], res_col[off:off + z])])
            off += z
    finally:
        for a in pinned:
            ga.host_unregister(a)
    parity = {"graph_matches_record": None, "sweep_vs_oracle_record": None}
    if golden is not None:
        parity["graph_matches_record"] = bool(edge_digest(rst, col) == golden["graph"]["digest"])
        gs = [list(x) for x in golden["stages"]]
        bad = [d[0] for d, g in zip(digests, gs) if d != g]
        parity["sweep_vs_oracle_record"] = {
            "stages": len(gs), "compared": min(len(gs), len(digests)), "equal": not bad and len(gs) == len(digests),
            "first_mismatch_k": bad[0] if bad else None,
            "what": "iteration count, stored entries and BLAKE2b digest of (row starts, columns) of every "
                    "k-truss the e2e sweep downloaded, against tests/golden/rmat18_sweep.json (CPU oracle)"}

    # ------------------------------------------------- support variants
    variants = {}
    default = {"warp_max_flops": 32768, "heavy_flops": 1 << 20, "ctas_per_sm": 0, "dot_chunk": 8}
    ga.apply_schedule(ctx, default)  # each variant with the default schedule
    for algo in ("msa", "mca", "heap", "dot", "hybrid", "tri"):
        ctx.work_counters(reset=True)
        ctx.flush_l2()
        ctx.timer_start()
        C = ga.mxm_masked(algo, A, A, A)
        ms = ctx.timer_stop()
        C.free()
        variants[algo] = {"ms": ms, "gflops": 2.0 * ctx.work_counters()["products"] / ms / 1e6}
    variants["autotune_ktruss"] = ga.autotune(ga.TUNE_KTRUSS, A)

    cpu = None
    if dist.rank == 0 and dist.world == 1 and not args.no_cpu_baseline:
        import oracle
        cpu, (R3, it3) = cpu_sample(oracle.Csr(m, m, rst, col, val), args.cpu_reps)
        C3, git3 = ga.ktruss(args.algo, A, 3)
        r3, c3, v3 = C3.download()
        C3.free()
        parity["k3_vs_oracle_live"] = bool(git3 == it3 and np.array_equal(r3, R3.rst) and np.array_equal(c3, R3.col)
                                           and np.array_equal(v3, R3.val))

    others = other_configs(ga, ctx, args, with_cpu=dist.world == 1) if not args.no_other_configs else None
    batch = serve = None
    if not args.no_other_configs:
        batch = batch_record(ga, ctx, args, dist)
        serve = serve_record(ga, ctx, args, dist)
    if others:
        parity["tc_er1000_bit_exact"] = others["tc_er1000"]["bit_exact"]
        if "parity" in others["bc_rmat20_64src"]:
            parity["bc_rmat20_64src_max_rel_err"] = others["bc_rmat20_64src"]["parity"]["max_rel_err"]
            parity["bc_rmat20_64src_within_1e-9"] = others["bc_rmat20_64src"]["parity"]["within_1e-9"]
    if batch:
        parity["batch_equal_to_plain"] = batch["plain"]["results_equal"]
    if serve:
        parity["serve_equal_to_plain"] = serve["results_equal"]

    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": dist.world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": t_max / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "int32", "data": "synthetic",
        "config": workload_config(args, m, nnz, kmax),
        "variant": args.algo, "schedule": None if schedule is None else
        {k: schedule[k] for k in ("algo", "warp_max_flops", "heavy_flops", "ctas_per_sm", "dot_chunk")},
        "parity": parity,
        "roofline": roofline, "cpu_baseline": cpu, "e2e": e2e,
        "gpu_launches": int(launches_per_step * args.steps), "clocks": clocks,
        "work": {"products_per_step": wc["products"] / args.steps,
                 "executed_products_per_step": wc["executed"] / args.steps, "k_max": kmax,
                 "support_products_k3": per_k.get(args.kmin, {}).get("products"),
                 "wedges_per_step": wc["wedges"] / args.steps, "triangles_per_step": wc["triangles"] / args.steps,
                 "frontier_edges_per_step": wc["front_edges"] / args.steps,
                 "frontier_probes_per_step": wc["front_probes"] / args.steps,
                 "frontier_triangles_per_step": wc["front_triangles"] / args.steps,
                 "note": "value counts 2 x the Gustavson products of the reference's C<C> = C*C for every "
                         "support product of every k (products_per_step): a reference-equivalent rate, not "
                         "arithmetic executed. The triangle-listing sweep lists the triangles of A once, and "
                         "again each time a k-truss keeps at most half of the listed graph's entries "
                         "(wedges_per_step rank-ordered lookups in all), and otherwise, k after k and "
                         "iteration after iteration, walks only the triangles of the edges it prunes "
                         "(frontier_*); the Gustavson forms execute executed_products_per_step products"},
        "kernel_profile": {"note": "one step with host-driven loops and CUDA events per launch (slower than "
                                   "the timed step); summed event time per kernel scope, ms",
                           "top": {k: round(v[1], 3) for k, v in
                                   sorted(prof["stats"].items(), key=lambda kv: -kv[1][1])[:14]}},
        "support_variants": variants,
        "other_configs": others,
        "batch": batch,
        "serve": serve,
    }
    ctx.close()
    return line


# ----------------------------------------------------------- batch workload
def knn_batch_sizes(count: int, seed: int):
    """Graph sizes of the batch workload: n ~ U[32, 4096], dim ~ U[4, 16]."""
    rng = np.random.default_rng(seed)
    return rng.integers(32, 4097, count).astype(np.int32), rng.integers(4, 17, count).astype(np.int32)


def batch_config(args, n, nnz):
    return {"workload": f"batched TC + 4-truss of {args.graphs} 30-NN graphs",
            "graphs": args.graphs, "vertices": int(n.sum()), "stored_entries": int(nnz),
            "graph": "n ~ U[32,4096], dim ~ U[4,16], points i.i.d. N(0,1), 30 nearest by Euclidean distance, "
                     f"symmetrised by union, seed {args.seed}",
            "variant": {"tc": args.batch_tc_algo, "ktruss": args.batch_algo}, "k": 4,
            "l2": "flushed between steps (256 MiB write)", "parallelism": "replicas only"}


def batch_record(ga, ctx, args, dist: Dist, steps: int = 3, warmup: int = 1, with_profile: bool = False,
                 cpu_budget_s: float = 5.0) -> dict:
    """Batched TC + 4-truss of args.graphs k-NN graphs (the block-diagonal
    union resident in HBM, GA_AUTO schedules tuned on it) against the plain
    per-graph form on the same GPU (ga_tc + ga_ktruss graph by graph on
    resident per-graph handles, MSA with the default schedule); results
    compared graph by graph; e2e uploads the union and downloads the
    results; the oracle port on a bounded sample of the graphs."""
    loops = 0 if args.host_loops else 1
    ctx.set_option(ga.OPT_DEVICE_LOOPS, loops)
    n, dim = knn_batch_sizes(args.graphs, args.seed)
    U, voff = ga.gen_knn_batch(ctx, n, dim, k=30, seed=args.seed + dist.rank)
    G = args.graphs
    kt_arg = args.batch_algo
    tc_arg = args.batch_tc_algo
    tuning = {}
    kt_algo, tc_algo = kt_arg, tc_arg
    if kt_arg == "auto":
        tuning["ktruss"] = ga.autotune(ga.TUNE_KTRUSS, U)
        kt_algo = tuning["ktruss"]["algo"]
    if tc_arg == "auto":
        tuning["tc"] = ga.autotune(ga.TUNE_TC, U)
        tc_algo = tuning["tc"]["algo"]

    def step():
        tcs = ga.batch_tc(tc_arg, U, voff)
        C, iters = ga.batch_ktruss(kt_arg, U, voff, 4)
        z = C.nnz
        C.free()
        return tcs, iters, z

    for _ in range(max(1, warmup)):
        ref = step()
    sampler = ClockSampler(dist.local_rank)
    dist.barrier()
    ctx.sync()
    sampler.start()
    step_ms = []
    for _ in range(steps):
        ctx.flush_l2()
        ctx.timer_start()
        out = step()
        step_ms.append(ctx.timer_stop())
    ctx.sync()
    clocks = sampler.stop()
    dist.barrier()
    stable = bool(np.array_equal(out[0], ref[0]) and np.array_equal(out[1], ref[1]) and out[2] == ref[2])
    t_max = dist.max(sum(step_ms))
    value = dist.sum(G * steps) / (t_max * 1e-3)
    prof = None
    if with_profile:
        prof = profile_step(ga, ctx, step, kt_algo, lambda: ctx.work_counters(), loops)
        prof["roofline"]["kernel_share_of_step"] = prof["kernel_ms"] / (sum(step_ms) / steps)

    # ------------------------------------------- per-graph plain launches
    rst, col, _ = U.download()
    blocks = ga.split_blocks(rst, col, voff)
    npl = G if args.plain_graphs <= 0 else min(G, args.plain_graphs)
    pick = np.sort(np.random.default_rng(args.seed + 1).choice(G, npl, replace=False)) if npl < G else np.arange(G)
    handles = [ga.Csr.upload(ctx, m_, m_, r, c, np.ones(len(c), np.int32)) for m_, r, c in (blocks[i] for i in pick)]
    plain_tc_algo = tc_arg if tc_arg != "auto" else "msa"
    plain_kt_algo = kt_arg if kt_arg != "auto" else "msa"
    for h in handles[:8]:
        ga.tc(plain_tc_algo, h, per_row=False)
        ga.ktruss(plain_kt_algo, h, 4)[0].free()
    ctx.sync()
    ctx.flush_l2()
    ctx.timer_start()
    plain_tc = np.zeros(npl, np.int64)
    plain_it = np.zeros(npl, np.int32)
    plain_nnz = 0
    for j, h in enumerate(handles):
        plain_tc[j] = ga.tc(plain_tc_algo, h, per_row=False)[0]
        C, plain_it[j] = ga.ktruss(plain_kt_algo, h, 4)
        plain_nnz += C.nnz
        C.free()
    plain_ms = ctx.timer_stop()
    same = bool(stable and np.array_equal(plain_tc, ref[0][pick]) and np.array_equal(plain_it, ref[1][pick])
                and (npl < G or plain_nnz == ref[2]))
    for h in handles:
        h.free()
    plain_value = dist.sum(npl) / (dist.max(plain_ms) * 1e-3)

    # ---------------------------------------------------------- e2e
    rst_h = np.ascontiguousarray(rst)
    col_h = np.ascontiguousarray(col)
    out_rst = np.empty(len(rst), np.int32)
    out_col = np.empty(len(col) + 1, np.int32)
    pinned = [rst_h, col_h, out_rst, out_col]
    for a in pinned:
        ga.host_register(a)
    try:
        e2e_ms, d2h = [], 0
        phases = {"upload": 0.0, "tc": 0.0, "ktruss": 0.0, "download": 0.0}
        dist.barrier()
        for _ in range(steps):
            ctx.flush_l2()
            ctx.timer_start()
            t0 = time.perf_counter()
            Ud = ga.Csr.upload(ctx, len(rst) - 1, len(rst) - 1, rst_h, col_h)  # values all 1, set on the device
            Ud.set_symmetric(1)  # k-NN graphs symmetrised by union
            t1 = time.perf_counter()
            tcs = ga.batch_tc(tc_arg, Ud, voff)
            t2 = time.perf_counter()
            C, iters = ga.batch_ktruss(kt_arg, Ud, voff, 4)
            z = C.nnz
            t3 = time.perf_counter()
            ga.lib().ga_csr_download(ctx.handle, C.handle, out_rst.ctypes.data_as(ga._p),
                                     out_col.ctypes.data_as(ga._p), None)
            C.free()
            Ud.free()
            e2e_ms.append(ctx.timer_stop())
            t4 = time.perf_counter()
            for key, x0, x1 in (("upload", t0, t1), ("tc", t1, t2), ("ktruss", t2, t3), ("download", t3, t4)):
                phases[key] += 1e3 * (x1 - x0) / steps
            d2h = tcs.nbytes + iters.nbytes + out_rst.nbytes + 4 * z
            same = same and bool(np.array_equal(tcs, ref[0]) and np.array_equal(iters, ref[1]) and z == ref[2])
        e2e_t = dist.max(sum(e2e_ms))
        e2e = {"value": dist.sum(G * steps) / (e2e_t * 1e-3), "unit": "graphs/s",
               "h2d_bytes_per_step": int(rst_h.nbytes + col_h.nbytes + voff.nbytes),
               "d2h_bytes_per_step": int(d2h), "ms_per_step": e2e_t / steps,
               "host_phases_ms": {k: round(v, 2) for k, v in phases.items()}}
    finally:
        for a in pinned:
            ga.host_unregister(a)
    cpu = None
    if dist.rank == 0 and dist.world == 1 and not args.no_cpu_baseline:
        cpu = batch_cpu_sample(blocks, args.seed, cpu_budget_s)
    return {"value": value, "unit": "graphs/s", "ms_per_step": t_max / steps, "steps": steps,
            "config": batch_config(args, n, len(col)), "clocks": clocks, "autotune": tuning,
            "variant": {"tc": tc_algo, "ktruss": kt_algo},
            "plain": {"value": plain_value, "unit": "graphs/s", "graphs_timed": npl, "ms": plain_ms,
                      "results_equal": same, "speedup": value / plain_value,
                      "form": f"ga_tc({plain_tc_algo}) + ga_ktruss({plain_kt_algo}) per graph, "
                              "resident per-graph handles"},
            "e2e": e2e, "e2e_speedup_vs_plain": e2e["value"] / plain_value, "cpu_baseline": cpu,
            "work": {"triangles": int(ref[0].sum()), "truss_entries": int(ref[2]), "max_iters": int(ref[1].max())},
            "profile": prof}


def run_batch(args, dist: Dist):
    """--workload batch: the batched record as the line's value."""
    import graphalgo_gb300 as ga
    from graphalgo_gb300 import build as gbuild
    gbuild.build()
    ctx = ga.Context(dist.local_rank)
    r = batch_record(ga, ctx, args, dist, steps=args.steps, warmup=args.warmup, with_profile=True,
                     cpu_budget_s=15.0)
    prof = r.pop("profile")
    line = {
        "metric": METRIC, "value": r["value"], "unit": "graphs/s", "n_gpus": dist.world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": r["ms_per_step"], "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "int32", "data": "synthetic", "config": r["config"],
        "roofline": prof["roofline"], "cpu_baseline": r["cpu_baseline"], "e2e": r["e2e"],
        "gpu_launches": int(prof["launches"] * args.steps), "clocks": r["clocks"], "autotune": r["autotune"],
        "variant": r["variant"], "plain": r["plain"],
        "work": dict(r["work"], products_per_step=prof["counters"]["products"]),
    }
    ctx.close()
    return line


def batch_cpu_sample(blocks, seed, budget_s: float = 5.0):
    """Oracle port (OpenMP, all host threads): TC + 4-truss graph by graph on
    a seeded sample of the batch's graphs until the time budget is spent."""
    import oracle
    oracle.build()
    threads = os.cpu_count() or 1
    oracle.set_num_threads(threads)
    order = np.random.default_rng(seed + 2).permutation(len(blocks))
    done, t = 0, 0.0
    for i in order:
        m_, r, c = blocks[i]
        A = oracle.Csr(m_, m_, r, c, np.ones(len(c), np.int32))
        t0 = time.perf_counter()
        oracle.tc_sandia(A)
        oracle.ktruss(A, 4)
        t += time.perf_counter() - t0
        done += 1
        if t >= budget_s:
            break
    return {"value": done / t, "unit": "graphs/s", "cores": threads, "kind": "port",
            "sample": f"{done} of {len(blocks)} graphs (seeded random order), TC + 4-truss each, {t:.1f} s"}


# ----------------------------------------------------------- serve workload
def serve_pool(args, ctx, ga):
    """Seeded graph pool: R-MAT (edge factor 16) at the given scales and
    30-NN Gaussian graphs (dim ~ U[4,16]) of the given sizes, host CSR."""
    pool = []
    for sc in [int(x) for x in args.rmat_scales.split(",") if x]:
        m, rst, col = ga.gen_rmat(sc, 16, 0.57, 0.19, 0.19, args.seed + sc)
        pool.append((f"rmat{sc}", m, rst, col))
    rng = np.random.default_rng(args.seed)
    for n in [int(float(x)) for x in args.knn_sizes.split(",") if x]:
        d = int(rng.integers(4, 17))
        U, voff = ga.gen_knn_batch(ctx, [n], [d], k=30, seed=args.seed + n)
        rst, col, _ = U.download()
        U.free()
        pool.append((f"knn{n}d{d}", n, rst, col))
    return pool


def serve_requests(args, pool, count):
    """Request types uniform over TC / k-truss (k ~ U{3..8}) / BC (32 seeded
    sources), graphs uniform over the pool."""
    import graphalgo_gb300 as ga
    rng = np.random.default_rng(args.seed + 7 + count)
    out = []
    for _ in range(count):
        g = int(rng.integers(len(pool)))
        t = int(rng.integers(3))
        m = pool[g][1]
        if t == ga.REQ_BC:
            out.append((t, g, 0, rng.choice(m, min(32, m), replace=False).astype(np.int32)))
        elif t == ga.REQ_KTRUSS:
            out.append((t, g, int(rng.integers(3, 9)), None))
        else:
            out.append((t, g, 0, None))
    return out


def serve_run(ga, pool, reqs, workers, coalesce, arrivals=None, algo="msa"):
    """Runs the requests through a server; arrivals (seconds from the start)
    or all at once. Returns latencies, makespan and results."""
    with ga.Server(0, workers=workers, coalesce=coalesce, tc_algo=algo, ktruss_algo=algo) as srv:
        for _, m, rst, col in pool:
            srv.add_graph(m, rst, col)
        ids = []
        t0 = time.perf_counter()
        for i, (t, g, k, src) in enumerate(reqs):
            if arrivals is not None:
                dt = t0 + arrivals[i] - time.perf_counter()
                if dt > 0:
                    time.sleep(dt)
            ids.append(srv.submit(t, g, k=k, sources=src, want_edges=(t == ga.REQ_KTRUSS)))
        res = [srv.wait(r, timeout=3600) for r in ids]
        st = srv.stats()
    bad = [r for r in res if r["status"] != ga.OK]
    if bad:
        raise RuntimeError(f"{len(bad)} requests failed: {bad[0]['error']}")
    lat = np.array([r["t_end"] - r["t_submit"] for r in res])
    span = max(r["t_end"] for r in res) - min(r["t_submit"] for r in res)
    d2h = 0
    for (t, g, _, _), r in zip(reqs, res):
        d2h += 8 if t == ga.REQ_TC else (8 * pool[g][1] if t == ga.REQ_BC else 4 * (pool[g][1] + 1 + r["nnz"]))
    return {"req_s": len(reqs) / span, "p50_ms": 1e3 * float(np.percentile(lat, 50)),
            "p99_ms": 1e3 * float(np.percentile(lat, 99)), "makespan_s": span, "stats": st, "results": res,
            "d2h_bytes": d2h}


def serve_digest(ga, reqs, res):
    """Per-request results reduced to comparable values."""
    out = []
    for (t, _, _, _), r in zip(reqs, res):
        if t == ga.REQ_TC:
            out.append(("tc", r["tc"]))
        elif t == ga.REQ_KTRUSS:
            out.append(("kt", r["iters"], r["nnz"], int(np.sum(r["col"], dtype=np.int64))))
        else:
            out.append(("bc", r["bc"]))
    return out


def serve_same(a, b):
    for x, y in zip(a, b):
        if x[0] == "bc":
            if not np.allclose(x[1], y[1], rtol=1e-9, atol=1e-9):
                return False
        elif x != y:
            return False
    return True


def serve_classes(ga, pool, reqs, plain, srv):
    """Per request class (type, graph): count, the plain form's summed
    service time (t_end - t_start, one request at a time: its share of the
    plain makespan) and p50 latency in both forms."""
    names = {ga.REQ_TC: "tc", ga.REQ_KTRUSS: "ktruss", ga.REQ_BC: "bc"}
    cls = {}
    for i, (t, g, _, _) in enumerate(reqs):
        cls.setdefault(f"{names[t]}:{pool[g][0]}", []).append(i)
    out = {}
    span = plain["makespan_s"]
    for key, idx in sorted(cls.items()):
        svc = sum(plain["results"][i]["t_end"] - plain["results"][i]["t_start"] for i in idx)
        lat_p = [plain["results"][i]["t_end"] - plain["results"][i]["t_submit"] for i in idx]
        lat_s = [srv["results"][i]["t_end"] - srv["results"][i]["t_submit"] for i in idx]
        out[key] = {"requests": len(idx), "plain_service_s": round(svc, 4),
                    "plain_share": round(svc / span, 4) if span else None,
                    "p50_ms_plain": round(1e3 * float(np.median(lat_p)), 2),
                    "p50_ms_server": round(1e3 * float(np.median(lat_s)), 2)}
    return out


def serve_mix(ga, args, pool, reqs, rates, tag):
    """One request mix on one pool: saturated (all queued at once) server
    against the plain form, then Poisson arrivals at multiples of the plain
    form's rate, p50/p99 of each."""
    al = args.serve_algo
    plain = serve_run(ga, pool, reqs, 1, False, algo=al)
    l0 = ga.kernel_launches()
    srv = serve_run(ga, pool, reqs, args.workers, True, algo=al)
    launches = ga.kernel_launches() - l0
    same = serve_same(serve_digest(ga, reqs, plain["results"]), serve_digest(ga, reqs, srv["results"]))
    sweep_ = []
    rng = np.random.default_rng(args.seed + 11)
    for f in rates:
        lam = f * plain["req_s"]
        arrivals = np.cumsum(rng.exponential(1.0 / lam, len(reqs)))
        row = {"rate_req_s": lam, "rate_x_plain": f}
        for name, w, c in (("server", args.workers, True), ("plain", 1, False)):
            r = serve_run(ga, pool, reqs, w, c, arrivals, algo=al)
            row[name] = {k: r[k] for k in ("req_s", "p50_ms", "p99_ms")}
            same = same and serve_same(serve_digest(ga, reqs, plain["results"]), serve_digest(ga, reqs, r["results"]))
        sweep_.append(row)
    return {"pool": tag, "graphs": [g[0] for g in pool], "requests": len(reqs),
            "server": {k: srv[k] for k in ("req_s", "p50_ms", "p99_ms", "makespan_s")},
            "plain": {k: plain[k] for k in ("req_s", "p50_ms", "p99_ms", "makespan_s")},
            "speedup": srv["req_s"] / plain["req_s"], "results_equal": same,
            "batched_calls": srv["stats"]["batched_calls"], "max_group": srv["stats"]["max_group"],
            "gpu_launches": int(launches), "poisson": sweep_, "classes": serve_classes(ga, pool, reqs, plain, srv),
            "d2h_bytes_per_request": srv["d2h_bytes"] / len(reqs),
            "h2d_bytes_per_request": sum(4 * len(x[3]) for x in reqs if x[3] is not None) / len(reqs)}


def serve_record(ga, ctx, args, dist: Dist, light_requests=None, full_requests=None, rates=(1.0, 2.0)) -> dict:
    """The request server against the plain sequential form (one worker, no
    batching), the same requests in both: the light mix (the pool's graphs of
    at most 2^20 stored entries: R-MAT 10-14 and k-NN 1e3 / 1e4, where
    per-request costs bound the rate) and the full pool (R-MAT 10-22, k-NN up
    to 1e6, where single heavy requests do), with a per-class breakdown."""
    light_requests = args.serve_requests if light_requests is None else light_requests
    full_requests = args.serve_full_requests if full_requests is None else full_requests
    t_pool = time.perf_counter()
    pool = serve_pool(args, ctx, ga)
    t_pool = time.perf_counter() - t_pool
    tuned = {}
    t_tune = time.perf_counter()
    if args.serve_algo == "auto":
        for name, m, rst, col in pool:
            A = ga.Csr.upload(ctx, m, m, rst, col, np.ones(len(col), np.int32))
            kt = ga.autotune(ga.TUNE_KTRUSS, A)
            tc = ga.autotune(ga.TUNE_TC, A)
            tuned[name] = {"ktruss": kt["algo"], "tc": tc["algo"]}
            A.free()
    t_tune = time.perf_counter() - t_tune
    light = [g for g in pool if len(g[3]) <= (1 << 20)]
    sampler = ClockSampler(dist.local_rank)
    sampler.start()
    out = {"unit": "req/s", "workers": args.workers, "variant": args.serve_algo, "tuned": tuned,
           "pool_build_s": t_pool, "tuning_s": t_tune,
           "graphs": {name: {"vertices": m, "stored_entries": len(col)} for name, m, _, col in pool}}
    # warm-up of both forms: a few requests of each kind on the small graphs
    warm = serve_requests(args, light, 12)
    serve_run(ga, light, warm, args.workers, True, algo=args.serve_algo)
    serve_run(ga, light, warm, 1, False, algo=args.serve_algo)
    if light and light_requests > 0:
        out["light_mix"] = serve_mix(ga, args, light, serve_requests(args, light, light_requests), rates, "light")
    if full_requests > 0:
        out["full_pool"] = serve_mix(ga, args, pool, serve_requests(args, pool, full_requests), rates[:1], "full")
    out["clocks"] = sampler.stop()
    lm = out.get("light_mix")
    out["value"] = lm["server"]["req_s"] if lm else out["full_pool"]["server"]["req_s"]
    out["speedup"] = lm["speedup"] if lm else out["full_pool"]["speedup"]
    out["results_equal"] = all(out[k]["results_equal"] for k in ("light_mix", "full_pool") if k in out)
    return out


def run_serve(args, dist: Dist):
    """--workload serve: the serving record, the light mix's server req/s as
    the value."""
    import graphalgo_gb300 as ga
    from graphalgo_gb300 import build as gbuild
    gbuild.build()
    ctx = ga.Context(dist.local_rank)
    r = serve_record(ga, ctx, args, dist, light_requests=args.requests, full_requests=args.requests,
                     rates=tuple(float(x) for x in args.rates.split(",") if x))
    main_mix = r.get("light_mix") or r["full_pool"]
    line = {
        "metric": METRIC, "value": r["value"], "unit": "req/s", "n_gpus": dist.world, "steps": args.requests,
        "warmup": 12, "ms_per_step": 1e3 / r["value"], "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "int32/f64", "data": "synthetic",
        "config": {"workload": f"serving {args.requests} requests (TC / k-truss k~U{{3..8}} / BC 32 sources) "
                               "on the light mix and on the full pool of resident graphs",
                   "workers": args.workers, "l2": "inputs resident; not flushed between requests",
                   "parallelism": "replicas only"},
        "roofline": None, "cpu_baseline": None,
        "e2e": {"value": r["value"], "unit": "req/s", "h2d_bytes_per_step": main_mix["h2d_bytes_per_request"],
                "d2h_bytes_per_step": main_mix["d2h_bytes_per_request"],
                "note": "requests submitted from the host, results (counts, BC scores, k-truss edge sets) "
                        "returned to host memory; graphs resident"},
        "gpu_launches": main_mix["gpu_launches"], "clocks": r["clocks"], "serve": r,
    }
    ctx.close()
    return line


# --------------------------------------------------------- reference arm
def write_mtx_pattern(path: str, m: int, i1: np.ndarray, j1: np.ndarray, symmetric: bool = True) -> int:
    """Matrix Market pattern file of the 1-based entries (i1, j1) in the given
    order, each index right-aligned in a fixed-width field; returns bytes."""
    width = len(str(m))
    ne = len(i1)
    buf = np.full((ne, 2 * width + 2), ord(" "), np.uint8)
    for k, arr in enumerate((np.asarray(i1, np.int64), np.asarray(j1, np.int64))):
        for d in range(width):
            digit = (arr // 10 ** d) % 10
            buf[:, k * (width + 1) + width - 1 - d] = np.where((arr >= 10 ** d) | (d == 0), 48 + digit, 32)
    buf[:, -1] = ord("\n")
    head = (f"%%MatrixMarket matrix coordinate pattern {'symmetric' if symmetric else 'general'}\n"
            f"{m} {m} {ne}\n").encode()
    with open(path, "wb") as f:
        f.write(head)
        f.write(buf.tobytes())
    return len(head) + buf.size


def run_ingest(args, dist: Dist):
    """Graph-file ingestion: a seeded R-MAT graph (scale --ingest-scale, edge
    factor 16) written as a symmetric pattern Matrix Market file (its lower
    triangle, column-major, as collection files are ordered), read by
    ga_read_mtx with the reference CLI's preparation (adjacency, lower-
    triangle symmetrisation) into a device CSR. value = file entries per
    second, wall clock of the call (file in the page cache, read, copied,
    tokenised, parsed and built on the device); device = the ingestion
    kernels' time (CUDA events). Parity: the CSR read back equals the
    generator's CSR bit for bit. cpu_baseline: the C port of the
    reference's reader and preparation (serial, as the reference's reader
    is) on the first 2M entries of the same file."""
    import graphalgo_gb300 as ga
    import oracle
    from graphalgo_gb300 import build as gbuild
    gbuild.build()
    ctx = ga.Context(dist.local_rank)
    m, rst, col = ga.gen_rmat(args.ingest_scale, args.edge_factor, 0.57, 0.19, 0.19, args.seed)
    rows = np.repeat(np.arange(m, dtype=np.int64), np.diff(rst))
    low = rows > col
    # column-major order of the lower triangle: by column, then row
    order = np.lexsort((rows[low], col[low]))
    i1, j1 = rows[low][order] + 1, col[low].astype(np.int64)[order] + 1
    tmpdir = tempfile.mkdtemp(prefix="ga_ingest_")
    path = os.path.join(tmpdir, "rmat.mtx")
    nbytes = write_mtx_pattern(path, m, i1, j1)
    flags = ga.EDGES_LOWER_SYMM | ga.EDGES_UNIT
    A, code = ga.read_mtx(ctx, path, flags)  # warm-up (page cache, allocator)
    gr, gc, _ = A.download()
    exact = bool(np.array_equal(gr, rst) and np.array_equal(gc, col))
    A.free()
    walls = []
    for _ in range(max(3, args.steps)):
        ctx.sync()
        t0 = time.perf_counter()
        A, _ = ga.read_mtx(ctx, path, flags)
        walls.append(time.perf_counter() - t0)
        A.free()
    ctx.set_option(ga.OPT_PROFILE, 1)
    ctx.reset_kernel_stats()
    A, _ = ga.read_mtx(ctx, path, flags)
    ctx.sync()
    phases = {k: round(v[1], 3) for k, v in ctx.kernel_stats().items()}
    ctx.set_option(ga.OPT_PROFILE, 0)
    A.free()
    wall = statistics.median(walls)
    ne = len(i1)
    # top-level regions only (edges_to_csr contains the edges_* and sort_rows regions)
    device_ms = sum(v for k, v in phases.items() if k in ("mtx_tokenize", "mtx_parse", "edges_to_csr"))
    peak, peak_kind = measured_peak_hbm()
    # algorithmic bytes: the text read once, the CSR written once
    alg_bytes = nbytes + 4 * (m + 1) + 8 * len(col)
    line = {"metric": "Matrix Market ingestion, file entries/s", "value": ne / wall / 1e6, "unit": "M entries/s",
            "n_gpus": 1, "steps": len(walls), "higher_is_better": True, "dtype": "int32", "data": "synthetic",
            "config": {"workload": f"rmat{args.ingest_scale} symmetric pattern .mtx ({nbytes / 1e6:.0f} MB, "
                                   f"{ne} entries) -> CSR with the CLI's preparation", "vertices": m,
                       "nnz": len(col)},
            "wall_ms": wall * 1e3, "device_ms": device_ms, "device_phases_ms": phases, "bit_exact": exact,
            "matcode": code.decode(),
            "roofline": {"bound": "hbm", "achieved": alg_bytes / (device_ms * 1e-3) / 1e9, "peak": peak,
                         "unit": "GB/s", "frac": alg_bytes / (device_ms * 1e-3) / 1e9 / peak, "traffic": None,
                         "peak_kind": peak_kind}}
    # CPU: the C port of the reference's reading on a bounded sample
    ns = min(ne, 2_000_000)
    spath = os.path.join(tmpdir, "sample.mtx")
    write_mtx_pattern(spath, m, i1[:ns], j1[:ns])
    t0 = time.perf_counter()
    S = oracle.read_mtx_cli(spath, True)
    cpu_s = time.perf_counter() - t0
    Ag, _ = ga.read_mtx(ctx, spath, flags)
    sr, sc, _ = Ag.download()
    Ag.free()
    line["cpu_baseline"] = {"value": ns / cpu_s / 1e6, "unit": "M entries/s", "cores": 1, "kind": "port",
                            "sample": f"first {ns} entries of the same file ({cpu_s:.1f} s)",
                            "sample_bit_exact": bool(np.array_equal(sr, S.rst) and np.array_equal(sc, S.col))}
    for f in (path, spath):
        os.unlink(f)
    os.rmdir(tmpdir)
    return line


def run_reference(args, dist: Dist):
    """The reference arm: the oracle port of the reference's k_truss
    (oracle/oracle.c, the parallel MSA product, OpenMP on every host core;
    pinned to the unmodified reference by tests/test_oracle_pin.py) on a
    bounded sample of the sweep, the k = 3 stage from A, per step. Nothing of
    the product is loaded: the graph comes from oracle.gen_rmat, the same
    graph as the product's generator (tests/test_host_logic.py), and k_max
    from the oracle's record of the whole sweep. Rank 0 only."""
    if dist.rank != 0:
        return None
    import oracle
    oracle.build()
    m, rst, col = oracle.gen_rmat(args.scale, args.edge_factor, 0.57, 0.19, 0.19, args.seed)
    A = oracle.Csr(m, m, rst, col, np.ones(len(col), np.int32))
    golden = load_sweep_golden(args)
    kmax = golden["stages"][-1][0] - 1 if golden else None
    threads = os.cpu_count() or 1
    oracle.set_num_threads(threads)
    prod = 0
    for _ in range(args.warmup):
        oracle.ktruss(A, 3)
    times = []
    for _ in range(args.steps):
        t0 = time.perf_counter()
        _, _, prod = oracle.ktruss(A, 3, with_products=True)
        times.append(time.perf_counter() - t0)
    total = sum(times)
    value = 2.0 * prod * args.steps / total / 1e9
    sample = (f"k=3 stage of the k-truss sweep from A ({prod:.4g} Gustavson products) per step, "
              f"oracle port of k_truss (parallel mxmm_msa) on {threads} host threads")
    return {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": dist.world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": 1e3 * total / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "int32", "data": "synthetic", "impl": "reference",
            "config": workload_config(args, m, len(col), kmax),
            "variant": "oracle port of the reference's k_truss with the parallel mxmm_msa",
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port", "sample": sample},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}


def main():
    args = parse_args()
    if args.case:
        run_case(args)
        return
    dist = Dist()
    try:
        if args.impl == "reference":
            line = run_reference(args, dist)
        elif args.workload == "batch":
            line = run_batch(args, dist)
        elif args.workload == "serve":
            line = run_serve(args, dist)
        elif args.workload == "ingest":
            line = run_ingest(args, dist)
        else:
            line = run_gpu(args, dist)
        if dist.rank == 0 and line is not None:
            print(json.dumps(line), flush=True)
    finally:
        dist.close()


if __name__ == "__main__":
    main()
