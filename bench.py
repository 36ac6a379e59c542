"""Benchmark: PQIVF search on a 10M x 96 unit-norm index, one GB300.

Workload (the 10M x 96 search configuration): 10,000,000 float32 vectors,
d = 96, drawn from a Gaussian mixture of 10,000 centers and L2-normalised;
coarse k = 16,384; 24 subquantizers x 256 codewords (4 dims each), uint8
codes; 10,000 queries from the same mixture; top-10; Euclidean. Data are
synthetic and seeded. The index is trained on the GPU before timing.

A step is one batched Search of all 10,000 queries (coarse probe, list scan,
exact rerank) with the queries already resident in HBM. `e2e` repeats the
metric through the host C-ABI call (queries copied host->device and results
device->host inside the timed region).

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl mine|reference]

Under torchrun each rank builds and searches its own replica (the path has no
exchange step), rank 0 prints one JSON line with the whole-job throughput.
"""
from __future__ import annotations

import argparse
import ctypes
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)

METRIC = "PQIVF queries/sec at recall@10>=0.9 (10M x 96)"
PEAKS_PATH = os.path.join(HERE, "MEASURED_PEAKS.json")


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="mine", choices=["mine", "reference"])
    ap.add_argument("--n", type=int, default=10_000_000)
    ap.add_argument("--dim", type=int, default=96)
    ap.add_argument("--centers", type=int, default=10_000)
    ap.add_argument("--sigma", type=float, default=0.5)
    ap.add_argument("--nlist", type=int, default=16384)
    ap.add_argument("--m", type=int, default=24)
    ap.add_argument("--pqk", type=int, default=256)
    ap.add_argument("--iters", type=int, default=10)
    ap.add_argument("--nq", type=int, default=10_000)
    ap.add_argument("--k", type=int, default=10)
    ap.add_argument("--nprobe", type=str, default="32,128")
    ap.add_argument("--recall-queries", type=int, default=1000)
    ap.add_argument("--target-recall", type=float, default=0.9)
    ap.add_argument("--cpu-seconds", type=float, default=10.0)
    ap.add_argument("--seed", type=int, default=1234)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--profile-region", action="store_true",
                    help="bracket the timed steps with cudaProfilerStart/Stop (for ncu --profile-from-start off)")
    ap.add_argument("--serve-seconds", type=float, default=8.0, help="served-stream phase length (0 = skip)")
    ap.add_argument("--serve-rate", type=str, default="2000,5000",
                    help="Poisson request arrivals per second, one served-stream phase per value")
    ap.add_argument("--serve-batch-probes", type=int, default=32768,
                    help="served stream: bound on a batch's summed nprobe (0 = none)")
    ap.add_argument("--knn", type=int, default=1, help="run the batched exact k-NN section (1M x 128, top-100)")
    ap.add_argument("--knn-n", type=int, default=1_000_000)
    ap.add_argument("--knn-nq", type=int, default=10_000)
    ap.add_argument("--knn-steps", type=int, default=3)
    ap.add_argument("--knn-only", action="store_true", help="run only the k-NN section and print its line")
    ap.add_argument("--train-bench", type=int, default=1,
                    help="run the training section (1M x 128, coarse 4096, 16 x 256 PQ, 25 iterations)")
    ap.add_argument("--train-only", action="store_true", help="run only the training section")
    ap.add_argument("--knn-variants", type=str,
                    default="squared_euclidean/tensor,cosine/tensor,manhattan/exact,squared_euclidean/exact,"
                            "cosine/exact")
    return ap.parse_args()


def log(*a):
    print(*a, file=sys.stderr, flush=True)


# ---------------------------------------------------------------------------
# data


def make_data(args, torch, dev):
    """Gaussian mixture of `centers` centers (N(0,1)), per-point noise sigma,
    rows L2-normalised. Queries come from the same mixture."""
    g = torch.Generator(device=dev)
    g.manual_seed(args.seed)
    centers = torch.randn(args.centers, args.dim, generator=g, device=dev)
    x = torch.empty(args.n, args.dim, device=dev)
    chunk = 1 << 20
    for s in range(0, args.n, chunk):
        e = min(args.n, s + chunk)
        lab = torch.randint(0, args.centers, (e - s,), generator=g, device=dev)
        v = centers[lab] + args.sigma * torch.randn(e - s, args.dim, generator=g, device=dev)
        x[s:e] = v / v.norm(dim=1, keepdim=True)
    lab = torch.randint(0, args.centers, (args.nq,), generator=g, device=dev)
    q = centers[lab] + args.sigma * torch.randn(args.nq, args.dim, generator=g, device=dev)
    q = q / q.norm(dim=1, keepdim=True)
    return x.contiguous(), q.contiguous()


def ground_truth(torch, x, q, k):
    """Exact top-k by Euclidean distance: FP32 GEMM candidates (top 64),
    re-ranked in FP64."""
    torch.backends.cuda.matmul.allow_tf32 = False
    xn = (x * x).sum(1)
    out = []
    cand_k = max(64, 4 * k)
    for s in range(0, q.shape[0], 256):
        qb = q[s:s + 256]
        best_d = None
        best_i = None
        for xs in range(0, x.shape[0], 1 << 21):
            xe = min(x.shape[0], xs + (1 << 21))
            d = xn[xs:xe][None, :] - 2.0 * qb @ x[xs:xe].T
            v, i = torch.topk(d, cand_k, dim=1, largest=False)
            i = i + xs
            if best_d is None:
                best_d, best_i = v, i
            else:
                cd = torch.cat([best_d, v], 1)
                ci = torch.cat([best_i, i], 1)
                vv, jj = torch.topk(cd, cand_k, dim=1, largest=False)
                best_d, best_i = vv, torch.gather(ci, 1, jj)
        cx = x[best_i].double()
        d64 = ((cx - qb.double()[:, None, :]) ** 2).sum(-1)
        o = torch.argsort(d64, dim=1)[:, :k]
        out.append(torch.gather(best_i, 1, o).cpu().numpy())
    return np.concatenate(out, 0)


def recall_at(ids, gt):
    k = gt.shape[1]
    return float(np.mean([len(set(ids[i, :k].tolist()) & set(gt[i].tolist())) / k for i in range(gt.shape[0])]))


# ---------------------------------------------------------------------------
# clocks


class ClockSampler:
    """nvidia-smi clocks and throttle reasons during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.gpu = gpu_index
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.gpu), "--query-gpu=" + self.FIELDS, "--format=csv,noheader,nounits",
                 "-lms", "100"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
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
        except Exception:
            self.proc.kill()
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            p = [s.strip() for s in ln.split(",")]
            if len(p) < 9:
                continue
            try:
                sm.append(float(p[1]))
                mx.append(float(p[2]))
            except ValueError:
                continue
            for nm, val in zip(names, p[5:9]):
                if val.lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(sm)}


# ---------------------------------------------------------------------------


def dist_setup(args):
    import torch

    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if ws > 1:
        import torch.distributed as dist

        os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
        backend = "nccl" if torch.cuda.is_available() else "gloo"
        if backend == "nccl":
            torch.cuda.set_device(local)
        dist.init_process_group(backend)
    return ws, rank, local


def barrier(ws):
    if ws > 1:
        import torch.distributed as dist

        dist.barrier()


def max_over_ranks(ws, v, torch, dev):
    if ws == 1:
        return v
    import torch.distributed as dist

    t = torch.tensor([v], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def build_index(args, x, torch):
    import hann_gb300 as hg

    t0 = time.perf_counter()
    xh = x.cpu().numpy()
    idx = hg.New(args.dim, hg.WithCoarseK(args.nlist), hg.WithNumSubquantizers(args.m), hg.WithPQK(args.pqk),
                 hg.WithKMeansIters(args.iters), hg.WithSeed(args.seed), hg.WithDevice(torch.cuda.current_device()))
    idx.BulkAddArrays(np.arange(args.n, dtype=np.int64), xh)
    t1 = time.perf_counter()
    idx.Train()
    torch.cuda.synchronize()
    t2 = time.perf_counter()
    log(f"bulk_add {t1 - t0:.1f}s train {t2 - t1:.1f}s")
    return idx, xh, t2 - t1


def cpu_baseline(args, idx, q_host, nprobe, mode_rows):
    """The oracle (C restatement of the reference's Search) timed on the host
    cores on a bounded sample of the same queries."""
    import oracle

    oracle.build()
    st = idx.export_state()
    lay = st["layout"]
    ix = oracle.OracleIndex.from_csr(lay["dimension"], lay["num_subquantizers"], lay["pq_k_eff"], st["coarse"],
                                     st["codebooks"], st["list_len"], st["ids"], st["vectors"], st["codes"])
    del st
    cores = os.cpu_count() or 1
    probe_n = min(64, q_host.shape[0])
    t0 = time.perf_counter()
    ix.search(q_host[:probe_n], args.k, nprobe, nthreads=cores)
    dt = time.perf_counter() - t0
    per_q = dt / probe_n
    n = int(min(q_host.shape[0], max(probe_n, args.cpu_seconds / max(per_q, 1e-9))))
    t0 = time.perf_counter()
    ix.search(q_host[:n], args.k, nprobe, nthreads=cores)
    dt = time.perf_counter() - t0
    return {"value": n / dt, "unit": "queries/s", "cores": cores, "kind": "port",
            "sample": f"{n} of {q_host.shape[0]} queries, nprobe {nprobe}, k {args.k}, parity (reconstructed-"
                      f"vector) distances, {cores} threads, {dt:.1f} s"}


def main():
    args = parse()
    import torch

    ws, rank, local = dist_setup(args)
    if args.impl == "reference" and rank != 0:
        return 0
    dev = torch.device("cuda", local)
    torch.cuda.set_device(dev)
    import __graft_entry__ as ge

    ge.build()
    import hann_gb300 as hg

    if args.knn_only:
        print(json.dumps({"knn": knn_section(args, torch, dev)}), flush=True)
        return 0
    if args.train_only:
        print(json.dumps({"train": train_section(args, torch, dev)}), flush=True)
        return 0
    x, q = make_data(args, torch, dev)
    idx, xh, train_s = build_index(args, x, torch)
    q_host = q.cpu().numpy()
    nr = min(args.recall_queries, args.nq)
    gt = ground_truth(torch, x, q[:nr], args.k)
    del x
    torch.cuda.empty_cache()

    # recall at each nprobe, exact-rerank mode and parity mode
    probes = [int(p) for p in args.nprobe.split(",")]
    rec = {}
    for npb in probes:
        for mode in (1, 0):
            ids, _, _ = idx.SearchBatch(q_host[:nr], args.k, nprobe=npb, mode=mode)
            rec[(npb, mode)] = recall_at(ids, gt)
    log("recall", {f"nprobe{a}_mode{b}": round(v, 4) for (a, b), v in rec.items()})
    choice = None
    for npb in probes:
        if rec[(npb, 1)] >= args.target_recall:
            choice = npb
            break
    if choice is None:
        choice = probes[-1]
    mode = 1

    if args.impl == "reference":
        cb = cpu_baseline(args, idx, q_host, choice, None)
        # steps: repeat bounded samples
        line = {"impl": "reference", "metric": METRIC, "value": cb["value"], "unit": "queries/s", "n_gpus": ws,
                "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1000.0 * 1.0 / cb["value"],
                "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
                "data": "synthetic", "config": workload_config(args, choice, mode, rec),
                "cpu_baseline": cb, "e2e": {"value": cb["value"], "unit": "queries/s", "h2d_bytes_per_step": 0,
                                            "d2h_bytes_per_step": 0}}
        print(json.dumps(line), flush=True)
        return 0

    # ------------------------------------------------------------------ timed
    nq = args.nq
    ids_d = torch.empty(nq, args.k, dtype=torch.int64, device=dev)
    dist_d = torch.empty(nq, args.k, dtype=torch.float64, device=dev)
    nout_d = torch.empty(nq, dtype=torch.int32, device=dev)
    # a stream of its own: the search is enqueued on it, and the events that
    # time it are recorded on it (a null handle would send the work to the
    # index's internal stream, which the events would not bracket)
    stream = torch.cuda.Stream(dev)
    torch.cuda.synchronize()

    def step():
        idx.SearchBatchDevice(q.data_ptr(), nq, args.k, choice, mode, ids_d.data_ptr(), dist_d.data_ptr(),
                              nout_d.data_ptr(), stream.cuda_stream)

    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize()
    sampler = ClockSampler(local)
    sampler.start()
    time.sleep(0.3)
    barrier(ws)
    torch.cuda.synchronize()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    if args.profile_region:
        torch.cuda.profiler.start()
    e0.record(stream)
    for _ in range(args.steps):
        step()
    e1.record(stream)
    if args.profile_region:
        torch.cuda.synchronize()
        torch.cuda.profiler.stop()
    torch.cuda.synchronize()
    barrier(ws)
    ms = e0.elapsed_time(e1)
    clocks = sampler.stop()
    # the same steps again with per-stage events (kept out of the timed region)
    idx.StageTimes()  # clear
    idx.SetProfiling(True)
    for _ in range(args.steps):
        step()
    torch.cuda.synchronize()
    idx.SetProfiling(False)
    stage_ms, launches, rows_scanned = idx.StageTimes()
    ms_max = max_over_ranks(ws, ms, torch, dev)
    value = ws * nq * args.steps / (ms_max / 1000.0)

    # sanity: the timed results equal the host-API results
    ids_t = ids_d.cpu().numpy()
    ids_h, _, _ = idx.SearchBatch(q_host[:256], args.k, nprobe=choice, mode=mode)
    if not np.array_equal(ids_t[:256], ids_h):
        log("WARNING: device-path ids differ from host-path ids")

    # e2e through the host C-ABI (pinned host buffers, copies inside the timed region)
    L = hg.load_library()
    qp = torch.from_numpy(q_host).pin_memory()
    kk = torch.full((nq,), args.k, dtype=torch.int32).pin_memory()
    npv = torch.full((nq,), choice, dtype=torch.int32).pin_memory()
    oi = torch.empty(nq, args.k, dtype=torch.int64).pin_memory()
    od = torch.empty(nq, args.k, dtype=torch.float64).pin_memory()
    on = torch.empty(nq, dtype=torch.int32).pin_memory()

    def e2e_step():
        rc = L.hann_pqivf_search_batch(idx.handle, ctypes.c_void_p(qp.data_ptr()), nq,
                                       ctypes.c_void_p(kk.data_ptr()), ctypes.c_void_p(npv.data_ptr()), args.k, mode,
                                       ctypes.c_void_p(oi.data_ptr()), ctypes.c_void_p(od.data_ptr()),
                                       ctypes.c_void_p(on.data_ptr()))
        assert rc == 0, L.hann_pqivf_last_error(idx.handle)

    for _ in range(max(1, args.warmup // 2)):
        e2e_step()
    torch.cuda.synchronize()
    barrier(ws)
    t0 = time.perf_counter()
    e2e_steps = max(3, args.steps // 2)
    for _ in range(e2e_steps):
        e2e_step()
    torch.cuda.synchronize()
    e2e_s = max_over_ranks(ws, time.perf_counter() - t0, torch, dev)
    e2e_value = ws * nq * e2e_steps / e2e_s
    h2d = nq * args.dim * 4 + nq * 4 * 2
    d2h = nq * args.k * (8 + 8) + nq * 4

    # the plain FP32 GPU path: the same search with every coarse distance on
    # the FP32 SIMT kernels (no tensor-core preselection); same results
    idx.SetPlainFP32(True)
    for _ in range(max(1, args.warmup // 2)):
        step()
    torch.cuda.synchronize()
    p0 = torch.cuda.Event(enable_timing=True)
    p1 = torch.cuda.Event(enable_timing=True)
    p0.record(stream)
    for _ in range(args.steps):
        step()
    p1.record(stream)
    torch.cuda.synchronize()
    plain_fp32_qps = nq * args.steps / (p0.elapsed_time(p1) / 1000.0)
    plain_same = bool(np.array_equal(ids_d.cpu().numpy(), ids_t))
    idx.SetPlainFP32(False)

    # one-query-per-call path (plain, one launch sequence per query)
    nplain = 200
    t0 = time.perf_counter()
    for i in range(nplain):
        idx.SearchBatch(q_host[i:i + 1], args.k, nprobe=choice, mode=mode)
    plain_qps = nplain / (time.perf_counter() - t0)

    # roofline of the scan kernel: algorithmic bytes = rows scanned (counted
    # by the kernel) x (M code bytes + the 4-byte per-row term)
    code_bytes = args.m + 4
    per_search = max(1, min(nq, (1 << 28) // args.nlist))
    scan_launches = args.steps * -(-nq // per_search)
    scan_ms = stage_ms[2] / scan_launches
    per_launch_bytes = rows_scanned / scan_launches * code_bytes
    achieved = per_launch_bytes / (scan_ms / 1000.0) / 1e9
    peak = 6782.4
    peak_src = "fallback"
    if os.path.exists(PEAKS_PATH):
        try:
            peak = float(json.load(open(PEAKS_PATH))["hbm_gbs"])
            peak_src = "measured"
        except Exception:
            pass

    served = None
    if args.serve_seconds > 0:
        served = []
        for rate in [float(r) for r in args.serve_rate.split(",") if r]:
            try:
                served.append(serve_stream(args, idx, q_host, gt, nr, rate))
                log("served", served[-1])
            except Exception as e:  # pragma: no cover
                log("served stream failed:", e)
                served.append({"offered_requests_per_s": rate, "error": str(e)})

    train = None
    if args.train_bench and rank == 0:
        try:
            train = train_section(args, torch, dev)
        except Exception as e:  # pragma: no cover
            log("train section failed:", e)
            train = {"error": str(e)}

    knn = None
    if args.knn and rank == 0:
        try:
            knn = knn_section(args, torch, dev)
        except Exception as e:  # pragma: no cover
            log("knn section failed:", e)
            knn = {"error": str(e)}

    cb = None
    if rank == 0 and not args.no_cpu_baseline:
        try:
            cb = cpu_baseline(args, idx, q_host, choice, None)
        except Exception as e:  # pragma: no cover
            log("cpu baseline failed:", e)
            cb = {"value": None, "unit": "queries/s", "cores": os.cpu_count(), "kind": "port", "sample": str(e)}

    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": "queries/s", "n_gpus": ws, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms_max / args.steps, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": workload_config(args, choice, mode, rec),
            "recall_at_10": rec[(choice, mode)],
            "stage_ms_per_step": [round(v / args.steps, 4) for v in stage_ms],
            "train_s": round(train_s, 2),
            "plain_one_query_per_call_qps": plain_qps,
            "plain_fp32_gpu_qps": plain_fp32_qps, "plain_fp32_same_ids": plain_same,
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                         "frac": achieved / peak, "traffic": scan_traffic(args, choice), "kernel": "scan_skew_kernel",
                         "bytes_per_launch": per_launch_bytes, "peak_source": peak_src},
            "cpu_baseline": cb,
            "e2e": {"value": e2e_value, "unit": "queries/s", "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h},
            "gpu_launches": launches,
            "clocks": clocks,
            "served_stream": served,
            "knn": knn,
            "train": train,
        }
        if served and "p50_ms" in served[0]:
            line["p50_ms"] = served[0]["p50_ms"]
            line["p99_ms"] = served[0]["p99_ms"]
        print(json.dumps(line), flush=True)
    idx.close()
    if ws > 1:
        import torch.distributed as dist

        dist.destroy_process_group()
    return 0


def train_section(args, torch, dev):
    """PQIVF training at scale: 1,000,000 x 128 float32 from a Gaussian
    mixture of 2,000 anisotropic clusters (per-cluster diagonal scales
    log-uniform in [0.05, 1]); coarse 4,096, 16 x 256 PQ (8 dims each), 25
    k-means iterations. Trains twice -- tensor-core assignment with exact
    boundary rescoring, and the plain FP32 SIMT assignment -- and reports
    wall time, time per iteration and the coarse inertia evaluated in FP64.
    Both must give the same index."""
    import hann_gb300 as hg

    n, dim, k, iters = 1_000_000, 128, 4096, 25
    g = torch.Generator(device=dev)
    g.manual_seed(args.seed + 11)
    centers = torch.randn(2000, dim, device=dev, generator=g) * 2.0
    scales = torch.exp(torch.rand(2000, dim, device=dev, generator=g) * (np.log(1.0) - np.log(0.05))
                       + np.log(0.05))
    lab = torch.randint(0, 2000, (n,), device=dev, generator=g)
    x = centers[lab] + torch.randn(n, dim, device=dev, generator=g) * scales[lab]
    xh = x.cpu().numpy()
    ids = np.arange(n, dtype=np.int64)
    out = {"workload": f"{n} x {dim} anisotropic Gaussian mixture (2000 clusters), coarse {k}, 16 x 256 PQ, "
                       f"{iters} k-means iterations"}
    states = {}
    for name, plain in (("tensor_core", False), ("plain_fp32", True)):
        idx = hg.New(dim, hg.WithCoarseK(k), hg.WithNumSubquantizers(16), hg.WithPQK(256),
                     hg.WithKMeansIters(iters), hg.WithPlainFP32(plain))
        idx.BulkAddArrays(ids, xh)
        torch.cuda.synchronize()
        t = time.perf_counter()
        idx.Train()
        torch.cuda.synchronize()
        el = time.perf_counter() - t
        st = idx.export_state()
        cent = torch.from_numpy(st["coarse"]).to(dev).double()
        lab_of = torch.from_numpy(np.repeat(np.arange(k), st["list_len"])).to(dev)
        rows = torch.from_numpy(st["ids"]).to(dev)
        d = x[rows].double() - cent[lab_of]
        inertia = float((d * d).sum().item())
        out[name] = {"train_s": round(el, 3), "s_per_iteration": round(el / iters, 4), "inertia_fp64": inertia}
        states[name] = st
        log("train", name, out[name])
        if not plain:
            # binary snapshot of this index: write, read back into a new
            # handle, and the same answers
            try:
                import tempfile
                with tempfile.TemporaryDirectory() as td:
                    path = os.path.join(td, "index.snap")
                    t = time.perf_counter()
                    idx.SaveSnapshot(path)
                    t_save = time.perf_counter() - t
                    size = os.path.getsize(path)
                    other = hg.New(dim)
                    t = time.perf_counter()
                    other.LoadSnapshot(path)
                    torch.cuda.synchronize()
                    t_load = time.perf_counter() - t
                qs_ = x[:256].cpu().numpy()
                same = all(np.array_equal(u, v) for u, v in zip(idx.SearchBatch(qs_, 10, nprobe=16, mode=1),
                                                                 other.SearchBatch(qs_, 10, nprobe=16, mode=1)))
                other.close()
                out["snapshot"] = {"bytes": size, "save_s": round(t_save, 3), "load_s": round(t_load, 3),
                                   "same_results": bool(same)}
                log("snapshot", out["snapshot"])
            except Exception as e:  # pragma: no cover
                out["snapshot"] = {"error": str(e)}
            # the reference's own format: Save / Load through the gob stream
            try:
                import tempfile
                with tempfile.TemporaryDirectory() as td:
                    path = os.path.join(td, "index.gob")
                    t = time.perf_counter()
                    with open(path, "wb") as f:
                        idx.Save(f)
                    t_save = time.perf_counter() - t
                    size = os.path.getsize(path)
                    other = hg.New(dim)
                    t = time.perf_counter()
                    with open(path, "rb") as f:
                        other.Load(f)
                    torch.cuda.synchronize()
                    t_load = time.perf_counter() - t
                qs_ = x[:256].cpu().numpy()
                same = all(np.array_equal(u, v) for u, v in zip(idx.SearchBatch(qs_, 10, nprobe=16, mode=1),
                                                                 other.SearchBatch(qs_, 10, nprobe=16, mode=1)))
                other.close()
                out["gob"] = {"bytes": size, "save_s": round(t_save, 3), "load_s": round(t_load, 3),
                              "same_results": bool(same)}
                log("gob", out["gob"])
            except Exception as e:  # pragma: no cover
                out["gob"] = {"error": str(e)}
        if not plain and args.serve_seconds > 0:
            # the served stream on this 1M x 128 index as well
            try:
                nq_s = 1000
                lab_q = torch.randint(0, 2000, (nq_s,), device=dev, generator=g)
                qs = centers[lab_q] + torch.randn(nq_s, dim, device=dev, generator=g) * scales[lab_q]
                gt = ground_truth(torch, x, qs, 10)
                out["served_stream_1Mx128"] = serve_stream(args, idx, qs.cpu().numpy(), gt, nq_s, 2000.0,
                                                           n_ids=n, seconds=min(4.0, args.serve_seconds))
                log("served 1Mx128", out["served_stream_1Mx128"])
            except Exception as e:  # pragma: no cover
                out["served_stream_1Mx128"] = {"error": str(e)}
        idx.close()
    a, b = states["tensor_core"], states["plain_fp32"]
    out["identical_index"] = bool(all(np.array_equal(a[key], b[key]) for key in ("coarse", "list_len", "ids",
                                                                                "codes")))
    return out


def knn_histogram_data(torch, dev, n, dim, seed):
    """Non-negative integers 0-255, 70% zeros, nonzeros geometric with mean
    20 (quantized-histogram-like vectors)."""
    g = torch.Generator(device=dev)
    g.manual_seed(seed)
    u = torch.rand(n, dim, device=dev, generator=g, dtype=torch.float64)
    geo = torch.floor(torch.log1p(-u) / np.log1p(-1.0 / 20.0)) + 1.0
    x = torch.clamp(geo, max=255.0).to(torch.float32)
    x[torch.rand(n, dim, device=dev, generator=g) < 0.7] = 0.0
    return x


def knn_section(args, torch, dev):
    """Batched exact k-NN: 1,000,000 x 128 histogram-like base, 10,000
    queries, top-100 under squared Euclidean, cosine (tensor-core screen +
    exact FP32 rescore, and the plain FP32 SIMT path) and Manhattan (FP32
    SIMT). Per variant: queries/s with inputs resident in HBM, recall@100
    and the largest relative distance error against an FP64 brute force of
    the first 100 queries, and for the screen how many queries fell back to
    the exact path."""
    import hann_gb300 as hg

    n, dim, nq, k = args.knn_n, 128, args.knn_nq, 100
    base = knn_histogram_data(torch, dev, n, dim, args.seed + 7)
    q = knn_histogram_data(torch, dev, nq, dim, args.seed + 8)
    idx = hg.KNN(base.cpu().numpy())
    ids = torch.empty(nq, k, dtype=torch.int64, device=dev)
    dist = torch.empty(nq, k, dtype=torch.float64, device=dev)
    stream = torch.cuda.Stream(dev)  # the k-NN runs and its timing events on one stream
    torch.cuda.synchronize()
    nr = min(100, nq)
    b64 = base.double()
    q64 = q[:nr].double()
    gt = {}
    for metric in ("squared_euclidean", "cosine", "manhattan"):
        if metric == "manhattan":
            d = torch.cdist(q64, b64, p=1)
        else:
            dot = q64 @ b64.T
            if metric == "squared_euclidean":
                d = (q64 * q64).sum(1, keepdim=True) - 2 * dot + (b64 * b64).sum(1)[None, :]
            else:
                qn = q64.norm(dim=1, keepdim=True)
                bn = b64.norm(dim=1)[None, :]
                den = qn * bn
                d = torch.where(den == 0, torch.ones_like(dot), 1 - torch.clamp(dot / torch.where(den == 0, 1, den),
                                                                                  -1, 1))
        # (distance, id) order: stable sort on distance keeps ids ascending
        dd, order = torch.sort(d, dim=1, stable=True)
        gt[metric] = (order[:, :k].cpu().numpy(), dd[:, :k].cpu().numpy())
    del b64
    out = {"workload": f"{n} x {dim} histogram-like (0-255, 70% zeros, geometric mean 20), {nq} queries, top-{k}"}
    variants = [tuple(v.split("/")) for v in args.knn_variants.split(",") if v]
    for metric, method in variants:
        def run():
            idx.search_device(q.data_ptr(), nq, k, ids.data_ptr(), dist.data_ptr(), metric, method,
                              stream.cuda_stream)
        before = idx.stats()
        run()
        torch.cuda.synchronize()
        t0 = torch.cuda.Event(enable_timing=True)
        t1 = torch.cuda.Event(enable_timing=True)
        t0.record(stream)
        for _ in range(args.knn_steps):
            run()
        t1.record(stream)
        torch.cuda.synchronize()
        ms = t0.elapsed_time(t1) / args.knn_steps
        after = idx.stats()
        got_i = ids[:nr].cpu().numpy()
        got_d = dist[:nr].cpu().numpy()
        gi, gd = gt[metric]
        rec = float(np.mean([len(set(got_i[i]) & set(gi[i])) / k for i in range(nr)]))
        rel = float(np.max(np.abs(got_d - gd) / np.maximum(np.abs(gd), 1e-30)))
        key = f"{metric}/{method}"
        out[key] = {"queries_per_s": nq / (ms / 1e3), "ms": round(ms, 3), "recall_at_100_vs_fp64": round(rec, 5),
                    "max_rel_dist_err_vs_fp64": rel,
                    "fallback_queries_per_run": (after["fallback_queries"] - before["fallback_queries"])
                    / (args.knn_steps + 1)}
        log("knn", key, out[key])
    # the screen must give exactly the exact path's answer
    for metric in ("squared_euclidean", "cosine") if len(variants) == 5 else ():
        idx.search_device(q.data_ptr(), nq, k, ids.data_ptr(), dist.data_ptr(), metric, "tensor", stream.cuda_stream)
        a = (ids.clone(), dist.clone())
        idx.search_device(q.data_ptr(), nq, k, ids.data_ptr(), dist.data_ptr(), metric, "exact", stream.cuda_stream)
        out[f"{metric}/tensor_equals_exact"] = bool(torch.equal(a[0], ids) and torch.equal(a[1], dist))
    # host (e2e) form of the screened squared Euclidean
    qh = q.cpu().numpy()
    idx.search(qh, k, "squared_euclidean", "tensor")
    t = time.perf_counter()
    idx.search(qh, k, "squared_euclidean", "tensor")
    out["squared_euclidean/tensor_e2e_queries_per_s"] = nq / (time.perf_counter() - t)
    # CPU: the oracle's restatement of the reference batch kernels on a sample
    if not args.no_cpu_baseline:
        import oracle

        oracle.build()
        bh = base.cpu().numpy()
        sample = 8
        t = time.perf_counter()
        oracle.knn(qh[:sample], bh, k, "squared_euclidean", nthreads=os.cpu_count() or 1)
        el = time.perf_counter() - t
        out["cpu_port_queries_per_s"] = sample / el
        out["cpu_port_sample"] = f"{sample} queries x {n} rows, squared Euclidean, {os.cpu_count()} threads"
    idx.close()
    return out


def scan_traffic(args, nprobe):
    """DRAM bytes (read + write) of one scan launch on this workload, from the
    1-pass ncu capture kept in profiles/ (ncu cannot run inside the bench);
    None when the capture was of another workload."""
    path = os.path.join(HERE, "profiles", "scan_skew_kernel_10Mx96_dram.json")
    try:
        rec = json.load(open(path))
        if (rec["n"], rec["dim"], rec["nlist"], rec["M"], rec["nq"], rec["nprobe"], rec["k"]) != \
                (args.n, args.dim, args.nlist, args.m, args.nq, nprobe, args.k):
            return None
        return float(rec["dram_bytes_read_per_launch"]) + float(rec["dram_bytes_write_per_launch"])
    except Exception:
        return None


def serve_stream(args, idx, q_host, gt, nr, rate, n_ids=None, seconds=None):
    """The served stream: Poisson arrivals at `rate` requests/s, each a
    block of 1-512 queries (log-uniform), k uniform in [1, 100], nprobe
    log-uniform in [8, 256]; BulkAdd of 1,000-vector chunks and Deletes of
    random ids, each at 1% of the request rate, applied beside the running
    batches. Queries are drawn from the first `nr` queries (which have ground
    truth). Reports p50/p99 latency (submit to result, the server's clock),
    queries/s, recall@10 over a sample of the requests with k >= 10, the
    relayout holds and how late the submitter kept to its schedule."""
    import threading
    import queue as qmod

    import hann_gb300 as hg

    rng = np.random.default_rng(args.seed + 7)
    dur = seconds or args.serve_seconds
    # The whole arrival schedule is drawn before the clock starts, and
    # Python's thread switch interval is shortened for the run, so the
    # submitting thread keeps to the schedule (a waiter holding the
    # interpreter for a whole 5 ms switch interval used to delay it, and the
    # delayed arrivals then came as one burst). Latency is the server's own,
    # from submit to completion.
    sched = []
    t = 0.0
    next_id = 50_000_000
    while True:
        t += rng.exponential(1.0 / rate)
        if t > dur:
            break
        u = rng.random()
        if u < 0.01:
            # random unit vectors: far from every query, so they do not
            # disturb the recall measured against the original ground truth
            chunk = rng.standard_normal((1000, q_host.shape[1])).astype(np.float32)
            chunk /= np.linalg.norm(chunk, axis=1, keepdims=True)
            sched.append((t, 1, (np.arange(next_id, next_id + 1000), chunk)))
            next_id += 1000
        elif u < 0.02:
            sched.append((t, 2, rng.integers(0, n_ids or args.n, 100)))
        else:
            nq = int(np.exp(rng.uniform(0, np.log(512))))
            k = int(rng.integers(1, 101))
            npb = int(np.exp(rng.uniform(np.log(8), np.log(256))))
            rows = rng.integers(0, nr, nq)
            sched.append((t, 0, (k, npb, rows)))
    srv = hg.Server(idx, slots=4, max_batch_queries=8192, max_k=100, max_nprobe=256, mode=1,
                    memory_budget=120 << 30, max_batch_probes=args.serve_batch_probes)
    pending = qmod.Queue()
    results = []

    def waiter():
        # results are copied out only for the requests the recall uses
        # (k >= 10, every fourth), so the interpreter stays free for the
        # submitting thread
        i = 0
        while True:
            item = pending.get()
            if item is None:
                return
            kind, tk, meta = item
            keep = kind == 0 and meta[1] >= 10 and i % 4 == 0
            i += kind == 0
            r = srv.wait(tk, timeout_ms=120000, results=keep)
            if keep:
                results.append((meta, r))

    old_switch = sys.getswitchinterval()
    sys.setswitchinterval(2e-4)
    ws = [threading.Thread(target=waiter, daemon=True) for _ in range(1)]
    for w in ws:
        w.start()
    late = []
    t0 = time.perf_counter()
    for ta, kind, payload in sched:
        while True:
            now = time.perf_counter() - t0
            if now >= ta:
                break
            time.sleep(min(ta - now, 0.0005))
        late.append(now - ta)
        if kind == 1:
            pending.put((1, srv.submit_add(*payload), None))
        elif kind == 2:
            pending.put((2, srv.submit_delete(payload), None))
        else:
            k, npb, rows = payload
            pending.put((0, srv.submit(q_host[rows], k, npb), (rows, k)))
    for _ in ws:
        pending.put(None)
    for w in ws:
        w.join()
    sys.setswitchinterval(old_switch)
    st = srv.stats()
    srv.stop()
    hits = tot = 0
    for (rows, k), (ids, dist, n, lat) in results:
        if k < 10:
            continue
        for j, r in enumerate(rows):
            hits += len(set(ids[j, :10].tolist()) & set(gt[r].tolist()))
            tot += 10
    return {"requests": int(st["requests"]), "queries": int(st["queries"]), "batches": int(st["batches"]),
            "mutations": int(st["mutations"]), "p50_ms": st["p50_ms"], "p99_ms": st["p99_ms"],
            "queries_per_s": st["queries_per_s"], "offered_requests_per_s": rate,
            "recall_at_10_k_ge_10": hits / tot if tot else None,
            "peak_admitted_bytes": int(st["peak_admitted_bytes"]), "relayouts": int(st["relayouts"]),
            "submit_late_ms_p99": round(1000.0 * float(np.percentile(late, 99)), 3) if late else None,
            "mutation_ms_total": round(st["mutation_ms"], 1), "relayout_drain_ms_total": round(st["drain_ms"], 1),
            "relayout_ms_total": round(st["relayout_ms"], 1), "relayout_max_ms": round(st["relayout_max_ms"], 1),
            "stream": "Poisson arrivals; 1-512 queries/request log-uniform; k U[1,100]; nprobe log-U[8,256]; "
                      "BulkAdd 1000-vector chunks and Deletes at 1% of the request rate; exact rerank",
            "max_batch_probes": args.serve_batch_probes}


def workload_config(args, nprobe, mode, rec):
    return {
        "workload": f"pqivf-search {args.n // 1_000_000}M x {args.dim} unit-norm Gaussian mixture "
                    f"({args.centers} centers, sigma {args.sigma}); coarse {args.nlist}; "
                    f"{args.m} x {args.pqk} PQ; {args.nq} queries; k {args.k}; nprobe {nprobe}; "
                    f"{'exact FP32 rerank of raw vectors' if mode == 1 else 'reference PQ distances'}",
        "n": args.n, "dim": args.dim, "nlist": args.nlist, "M": args.m, "pq_k": args.pqk, "nq": args.nq,
        "k": args.k, "nprobe": nprobe, "mode": "exact_rerank" if mode == 1 else "parity",
        "recall_by_nprobe": {f"{a}/{'exact' if b == 1 else 'pq'}": round(v, 4) for (a, b), v in rec.items()},
        "l2": f"inputs larger than L2 ({args.n * (2 * args.m) / 1e6:.0f} MB of scan words + "
              f"{args.n * args.dim * 4 / 1e9:.2f} GB raw vectors), no flush",
    }


if __name__ == "__main__":
    sys.exit(main())
