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
    ap.add_argument("--serve-seconds", type=float, default=5.0, help="served-stream phase length (0 = skip)")
    ap.add_argument("--serve-rate", type=str, default="2000,5000,10000,20000",
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
    ap.add_argument("--export-index", type=str, default="",
                    help="build the search index, write its state and the queries to this directory, exit "
                         "(the reference arm runs this in a child process so that its own process maps no "
                         "library of this repository)")
    ap.add_argument("--cpu-step-seconds", type=float, default=1.0,
                    help="reference arm: CPU seconds per step (each step a sample of the queries)")
    ap.add_argument("--config1", type=int, default=1,
                    help="run the plain 20k x 128 PQIVF section (train + search, GPU and CPU oracle)")
    ap.add_argument("--train-oracle-iters", type=int, default=2,
                    help="k-means iterations of the oracle's inertia check on the 1M x 128 training shape")
    ap.add_argument("--adc-tables", default="fixed16", choices=["fixed16", "fp16", "fp32"],
                    help="the table scan's lookup tables in the timed steps")
    ap.add_argument("--autotune", type=int, default=1,
                    help="run the scan autotuner (table scan or list-major scan by nprobe) before the timed steps")
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


def compare_results(g_ids, g_d, g_n, o_ids, o_d, o_n, rel=1e-5):
    """Parity of two result sets under the bar of the tests: counts equal,
    distances within `rel` relative, ids equal except inside ties (an id
    may differ only where the two distances it competes at lie within rel).
    Returns counts of the queries that break each part."""
    g_n = np.asarray(g_n)
    o_n = np.asarray(o_n)
    count_mismatch = int((g_n != o_n).sum())
    id_bad = 0
    max_rel = 0.0
    for i in range(len(g_n)):
        c = int(min(g_n[i], o_n[i]))
        gd = np.asarray(g_d[i][:c], np.float64)
        od = np.asarray(o_d[i][:c], np.float64)
        if c:
            max_rel = max(max_rel, float(np.max(np.abs(gd - od) / np.maximum(np.abs(od), 1e-12))))
        gi, oi = list(g_ids[i][:c]), list(o_ids[i][:c])
        for j in range(c):
            if gi[j] == oi[j]:
                continue
            if gi[j] in oi:
                jj = oi.index(gi[j])
                ok = abs(od[jj] - od[j]) <= rel * max(abs(od[j]), 1e-12) + 1e-12
            else:
                ok = abs(gd[j] - od[c - 1]) <= rel * max(abs(od[c - 1]), 1e-12) + 1e-12
            if not ok:
                id_bad += 1
                break
    return {"queries": int(len(g_n)), "count_mismatches": count_mismatch,
            "id_mismatches_outside_ties": id_bad, "max_rel_dist_err": max_rel}


def oracle_index_from_state(st):
    import oracle

    lay = st["layout"]
    return oracle.OracleIndex.from_csr(lay["dimension"], lay["num_subquantizers"], lay["pq_k_eff"], st["coarse"],
                                       st["codebooks"], st["list_len"], st["ids"], st["vectors"], st["codes"])


def rerank_depth(k, mode):
    """Candidates the GPU reranks per query (the library's automatic depth):
    k + 32 in parity mode, max(4k, 64) in exact-rerank mode, rounded up to 32."""
    r = k + 32 if mode == 0 else max(4 * k, 64)
    return (r + 31) // 32 * 32


def cpu_legs(args, idx, q_host, nprobe, gpu_parity, gpu_exact):
    """The oracle over every query of the step, on all host cores: the
    reference's Search (parity mode: reconstructed-vector PQ distances) and
    the same search with the GPU's exact rerank of the best candidates.
    Each is timed, and the GPU's results for the same queries are compared
    with it. Returns (cpu_baseline, parity)."""
    import oracle

    oracle.build()
    oracle.set_tier(oracle.TIER_NEON)
    ix = oracle_index_from_state(idx.export_state())
    cores = os.cpu_count() or 1
    nq = q_host.shape[0]
    t0 = time.perf_counter()
    o_par = ix.search(q_host, args.k, nprobe, nthreads=cores)
    t_par = time.perf_counter() - t0
    R = rerank_depth(args.k, 1)
    t0 = time.perf_counter()
    o_ex = ix.search(q_host, args.k, nprobe, nthreads=cores, rerank=R)
    t_ex = time.perf_counter() - t0
    parity = {"reference_pq_distances": compare_results(*gpu_parity, *o_par[:3]),
              "exact_rerank": compare_results(*gpu_exact, *o_ex[:3]),
              "what": f"GPU results of all {nq} queries of the step (nprobe {nprobe}, k {args.k}) against the "
                      "oracle's on the same exported index: counts, ids outside 1e-5-relative ties, "
                      "largest relative distance error"}
    cb = {"value": nq / t_ex, "unit": "queries/s", "cores": cores, "kind": "port",
          "sample": f"all {nq} queries of the step, nprobe {nprobe}, k {args.k}, the reference's Search "
                    f"restated in C (NEON summation order) + exact FP32 rerank of the best {R} candidates "
                    f"(the GPU arm's mode), {cores} threads, {t_ex:.1f} s",
          "parity_mode_queries_per_s": nq / t_par,
          "parity_mode_sample": f"all {nq} queries, the reference's Search alone (PQ distances), {t_par:.1f} s"}
    return cb, parity


def export_index(args):
    """Child process of the reference arm: builds the 10M x 96 index on the
    GPU (the CPU cannot train it in minutes), picks nprobe from recall as the
    GPU arm does, and writes the index state, the queries and the ground
    truth as .npy files to args.export_index."""
    import torch

    dev = torch.device("cuda", 0)
    torch.cuda.set_device(dev)
    import __graft_entry__ as ge

    ge.build()
    x, q = make_data(args, torch, dev)
    idx, _, _ = build_index(args, x, torch)
    q_host = q.cpu().numpy()
    nr = min(args.recall_queries, args.nq)
    gt = ground_truth(torch, x, q[:nr], args.k)
    del x
    choice, rec = pick_nprobe(args, idx, q_host, gt, nr)
    st = idx.export_state()
    out = args.export_index
    lay = st["layout"]
    for key in ("coarse", "codebooks", "list_len", "ids", "vectors"):
        np.save(os.path.join(out, key + ".npy"), np.ascontiguousarray(st[key]))
    np.save(os.path.join(out, "codes.npy"), np.ascontiguousarray(st["codes"], dtype=np.uint8))
    np.save(os.path.join(out, "queries.npy"), q_host)
    np.save(os.path.join(out, "gt.npy"), gt)
    meta = {"dim": lay["dimension"], "M": lay["num_subquantizers"], "pq_k": lay["pq_k_eff"], "choice": choice,
            "recall_gpu": {f"{a}/{'exact' if b == 1 else 'pq'}": v for (a, b), v in rec.items()}}
    json.dump(meta, open(os.path.join(out, "meta.json"), "w"))
    idx.close()
    return 0


def pick_nprobe(args, idx, q_host, gt, nr):
    """Recall@10 at each nprobe in both modes; the first nprobe whose
    exact-rerank recall reaches the target (else the largest)."""
    probes = [int(p) for p in args.nprobe.split(",")]
    rec = {}
    for npb in probes:
        for mode in (1, 0):
            ids, _, _ = idx.SearchBatch(q_host[:nr], args.k, nprobe=npb, mode=mode)
            rec[(npb, mode)] = recall_at(ids, gt)
    log("recall", {f"nprobe{a}_mode{b}": round(v, 4) for (a, b), v in rec.items()})
    choice = next((p for p in probes if rec[(p, 1)] >= args.target_recall), probes[-1])
    return choice, rec


def reference_arm(args):
    """The reference's CPU path on the host cores: the oracle's restatement
    of pqivf Search (C, NEON summation order) over the same index, timed in
    steps of a bounded query sample. The index is built by a child process
    (--export-index) and read back from files, so this process loads no
    library of this repository."""
    import shutil
    import tempfile

    import oracle

    oracle.build()
    oracle.set_tier(oracle.TIER_NEON)
    td = tempfile.mkdtemp(prefix="hann_ref_")
    try:
        cmd = [sys.executable, os.path.abspath(__file__), "--export-index", td] + [
            a for a in sys.argv[1:] if not a.startswith("--impl") and a != "reference"]
        env = {k: v for k, v in os.environ.items() if k not in ("RANK", "WORLD_SIZE", "LOCAL_RANK")}
        t0 = time.perf_counter()
        subprocess.run(cmd, check=True, env=env, stdout=subprocess.DEVNULL)
        build_s = time.perf_counter() - t0
        meta = json.load(open(os.path.join(td, "meta.json")))
        ld = lambda name: np.load(os.path.join(td, name + ".npy"))  # noqa: E731
        ix = oracle.OracleIndex.from_csr(meta["dim"], meta["M"], meta["pq_k"], ld("coarse"), ld("codebooks"),
                                         ld("list_len"), ld("ids"), ld("vectors"), ld("codes"))
        q_host = ld("queries")
        gt = ld("gt")
    finally:
        shutil.rmtree(td, ignore_errors=True)
    choice = int(meta["choice"])
    cores = os.cpu_count() or 1
    R = rerank_depth(args.k, 1)
    nq = q_host.shape[0]
    # calibrate the step: about cpu_step_seconds of CPU work
    t0 = time.perf_counter()
    ix.search(q_host[:256], args.k, choice, nthreads=cores, rerank=R)
    per_q = (time.perf_counter() - t0) / 256
    S = int(max(256, min(nq, args.cpu_step_seconds / max(per_q, 1e-9))))
    pos = 0

    def step():
        nonlocal pos
        rows = (np.arange(S) + pos) % nq
        pos = (pos + S) % nq
        t = time.perf_counter()
        ix.search(q_host[rows], args.k, choice, nthreads=cores, rerank=R)
        return time.perf_counter() - t

    for _ in range(args.warmup):
        step()
    times = [step() for _ in range(args.steps)]
    qps = S * len(times) / sum(times)
    nr = gt.shape[0]
    ids_ex, _, _, _ = ix.search(q_host[:nr], args.k, choice, nthreads=cores, rerank=R)
    t0 = time.perf_counter()
    ids_par, _, _, _ = ix.search(q_host[:nr], args.k, choice, nthreads=cores)
    par_qps = nr / (time.perf_counter() - t0)
    rec = {"exact_rerank": recall_at(ids_ex, gt), "reference_pq_distances": recall_at(ids_par, gt)}
    sample = (f"{S} queries per step of the {nq}-query workload (rotating), nprobe {choice}, k {args.k}: "
              f"the reference's Search restated in C (NEON summation order) with the GPU arm's exact FP32 rerank "
              f"of the best {R} candidates, {cores} threads; ms_per_step is scaled to {nq} queries")
    line = {"impl": "reference", "metric": METRIC, "value": qps, "unit": "queries/s", "n_gpus": 1,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1000.0 * nq / qps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic", "config": workload_config(args, choice, 1),
            "recall_at_10": rec,
            "cpu_baseline": {"value": qps, "unit": "queries/s", "cores": cores, "kind": "port", "sample": sample},
            "parity_mode_queries_per_s": par_qps,
            "parity_mode_sample": f"first {nr} queries, the reference's Search alone (PQ distances)",
            "index_build": f"trained on the GPU by a child process ({build_s:.0f} s incl. data and ground truth), "
                           "read back from files; only Search is timed",
            "e2e": {"value": qps, "unit": "queries/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)
    return 0


def main():
    args = parse()
    if args.export_index:
        return export_index(args)
    import torch

    ws, rank, local = dist_setup(args)
    if args.impl == "reference":
        # rank 0 alone runs the CPU arm; the index comes from a child process
        return reference_arm(args) if rank == 0 else 0
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

    idx.SetADCTables(args.adc_tables)
    # the scan autotuner: times the table scan and the list-major scan at
    # nprobe 8..256 on the workload's queries and routes each nprobe to the
    # faster (results in parity mode do not depend on it)
    tune = None
    if args.autotune:
        t0 = time.perf_counter()
        tune = idx.AutotuneScan(q_host[:min(args.nq, 10000)], args.k, mode=1)
        tune["seconds"] = round(time.perf_counter() - t0, 2)
        log("autotune", tune)

    # recall at each nprobe, exact-rerank mode and parity mode
    choice, rec = pick_nprobe(args, idx, q_host, gt, nr)
    mode = 1

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
    plain_ids = ids_d.cpu().numpy()
    plain_same = float(np.mean([len(set(plain_ids[i].tolist()) & set(ids_t[i].tolist())) / args.k
                                for i in range(nq)]))
    plain_recall = recall_at(plain_ids[:nr], gt)
    idx.SetPlainFP32(False)

    # one-query-per-call path (plain, one launch sequence per query)
    nplain = 200
    t0 = time.perf_counter()
    for i in range(nplain):
        idx.SearchBatch(q_host[i:i + 1], args.k, nprobe=choice, mode=mode)
    plain_qps = nplain / (time.perf_counter() - t0)

    # the other nprobe values of the workload, timed the same way
    by_nprobe = {}
    for npb in [int(p) for p in args.nprobe.split(",")]:
        def step_np():
            idx.SearchBatchDevice(q.data_ptr(), nq, args.k, npb, mode, ids_d.data_ptr(), dist_d.data_ptr(),
                                  nout_d.data_ptr(), stream.cuda_stream)
        for _ in range(args.warmup):
            step_np()
        torch.cuda.synchronize()
        n0 = torch.cuda.Event(enable_timing=True)
        n1 = torch.cuda.Event(enable_timing=True)
        n0.record(stream)
        for _ in range(args.steps):
            step_np()
        n1.record(stream)
        torch.cuda.synchronize()
        ms_np = n0.elapsed_time(n1) / args.steps
        by_nprobe[str(npb)] = {"queries_per_s": nq / (ms_np / 1e3), "ms_per_step": ms_np,
                               "recall_at_10_exact_rerank": rec[(npb, 1)],
                               "recall_at_10_reference_pq_distances": rec[(npb, 0)]}
    log("by nprobe", by_nprobe)

    # the lookup tables of the table scan (FP32 against FP16 and 16-bit fixed
    # point) at the chosen nprobe: the step time and recall in exact-rerank
    # mode, and in parity mode the step time and the queries whose top k the
    # 16-bit screen could not prove (scanned again with FP32 tables)
    adc_tables = {}
    for kind in ("fixed16", "fp16", "fp32"):
        idx.SetADCTables(kind)
        row = {}
        for md in (1, 0):
            def step_kind():
                idx.SearchBatchDevice(q.data_ptr(), nq, args.k, choice, md, ids_d.data_ptr(), dist_d.data_ptr(),
                                      nout_d.data_ptr(), stream.cuda_stream)
            for _ in range(args.warmup):
                step_kind()
            torch.cuda.synchronize()
            r0 = idx.ADCRedos()
            k0 = torch.cuda.Event(enable_timing=True)
            k1 = torch.cuda.Event(enable_timing=True)
            k0.record(stream)
            for _ in range(args.steps):
                step_kind()
            k1.record(stream)
            torch.cuda.synchronize()
            tag = "exact_rerank" if md == 1 else "parity"
            row[f"{tag}_ms_per_step"] = k0.elapsed_time(k1) / args.steps
            row[f"{tag}_recall_at_10"] = recall_at(ids_d[:nr].cpu().numpy(), gt)
            if md == 0:
                row["parity_fp32_rescans_per_step"] = (idx.ADCRedos() - r0) / args.steps
        adc_tables[kind] = row
    idx.SetADCTables(args.adc_tables)
    log("lookup tables", adc_tables)

    # roofline of the scan: algorithmic bytes = rows scanned (counted by the
    # kernel, per (query, list)) x M code bytes, over the scan stage's event
    # time (the scan kernel and the selection kernel that follows it)
    code_bytes = args.m
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

    fp8 = None
    if rank == 0:
        try:
            fp8 = fp8_probe_study(torch, dev, idx.export_state()["coarse"], q, choice)
            log("fp8 probe study", fp8)
        except Exception as e:  # pragma: no cover
            fp8 = {"error": str(e)}

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
    parity = None
    if rank == 0 and not args.no_cpu_baseline:
        try:
            gpu_par = idx.SearchBatch(q_host, args.k, nprobe=choice, mode=0)
            gpu_ex = idx.SearchBatch(q_host, args.k, nprobe=choice, mode=1)
            cb, parity = cpu_legs(args, idx, q_host, choice, gpu_par, gpu_ex)
            log("cpu baseline", cb)
            log("parity", parity)
        except Exception as e:  # pragma: no cover
            log("cpu baseline failed:", e)
            cb = {"value": None, "unit": "queries/s", "cores": os.cpu_count(), "kind": "port", "sample": str(e)}

    config1 = None
    if args.config1 and rank == 0:
        try:
            config1 = config1_section(args, torch, dev)
        except Exception as e:  # pragma: no cover
            log("config1 section failed:", e)
            config1 = {"error": str(e)}

    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": "queries/s", "n_gpus": ws, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms_max / args.steps, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "u8 codes, int16 tables, f32 rerank", "data": "synthetic",
            "config": workload_config(args, choice, mode),
            "recall_at_10": rec[(choice, mode)],
            "recall_by_nprobe": {f"{a}/{'exact' if b == 1 else 'pq'}": round(v, 4) for (a, b), v in rec.items()},
            "by_nprobe": by_nprobe,
            "parity": parity,
            "stage_ms_per_step": [round(v / args.steps, 4) for v in stage_ms],
            "train_s": round(train_s, 2),
            "plain_one_query_per_call_qps": plain_qps,
            "plain_fp32_gpu_qps": plain_fp32_qps, "plain_fp32_recall_at_10": plain_recall,
            "plain_fp32_id_overlap": plain_same,
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                         "frac": achieved / peak, "traffic": scan_traffic(args, choice),
                         "kernel": f"scan_adc_kernel ({args.adc_tables} tables) + scan_select_kernel: the list "
                                   "scan and its candidate selection, timed together by the scan stage's events",
                         "bytes_per_launch": per_launch_bytes, "peak_source": peak_src},
            "adc_tables": adc_tables,
            "autotune": tune,
            "fp8_probe_study": fp8,
            "cpu_baseline": cb,
            "e2e": {"value": e2e_value, "unit": "queries/s", "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h},
            "gpu_launches": launches,
            "clocks": clocks,
            "served_stream": served,
            "knn": knn,
            "train": train,
            "config1": config1,
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


def fp8_probe_study(torch, dev, coarse, q, nprobe, nq=2000):
    """The FP8-e4m3 coarse-probe screen measured against the BF16 one on the
    workload's own centroids and queries. The screen ranks centroids by
    s~ = ||b||^2 - 2 <a~, b~> and the exact rescore must cover every centroid
    with s~ <= T~ + 2 eps (T~ the nprobe-th smallest s~, eps the bound of the
    operands' rounding: 2 (|a - a~| max|b| + |a~| max|b - b~|), plus FP32
    accumulation). The band size is the exact work each screen leaves; FP8
    rounds each operand to 3 mantissa bits (per-vector scale to e4m3's range)
    against BF16's 8."""
    a = q[:nq].double()
    b = torch.as_tensor(coarse, device=dev).double()
    bn2 = (b * b).sum(1)
    out = {}

    def rounded(x, kind):
        if kind == "bf16":
            return x.float().bfloat16().double()
        scale = x.abs().amax(1, keepdim=True).clamp_min(1e-30) / 448.0
        return (x.float() / scale.float()).to(torch.float8_e4m3fn).double() * scale

    for kind in ("bf16", "fp8_e4m3"):
        at, bt = rounded(a, kind), rounded(b, kind)
        s_t = bn2[None, :] - 2.0 * (at @ bt.T)
        ar = (a - at).norm(dim=1)
        an = at.norm(dim=1)
        bmax = b.norm(dim=1).max()
        brmax = (b - bt).norm(dim=1).max()
        kp = a.shape[1]
        eps = 2.0 * (ar * bmax + an * brmax) + 2.0 * kp * 2.0 ** -22 * (an * (bmax + brmax))
        thr = s_t.kthvalue(nprobe, dim=1).values + 2.0 * eps
        band = (s_t <= thr[:, None]).sum(1).double()
        out[kind] = {"band_mean": round(float(band.mean()), 1), "band_p99": float(band.quantile(0.99)),
                     "band_max": int(band.max()), "operand_rel_err": round(float((ar / a.norm(dim=1)).mean()), 6)}
    out["what"] = (f"{nq} queries x {b.shape[0]} centroids, nprobe {nprobe}: centroids the exact rescore must "
                   "cover after each screen (the band), and the mean relative rounding error of the queries")
    return out


def config1_section(args, torch, dev):
    """Plain PQIVF, the reference's CPU-sized case: 20,000 x 128 float32 from
    a Gaussian mixture of 64 centres (N(0,1), sigma 0.3); coarse 64, 8 x 256
    PQ, 10 k-means iterations from one seeded init given to both sides; 1,000
    queries from the same mixture, top-10, default nprobe 3. GPU and oracle
    each train and search; reported: train seconds, batched queries/s, one-
    query-per-call p50/p99, recall@10 against FP64 brute force, coarse
    inertia of both trainings (FP64) and the GPU search against the oracle
    on the GPU-trained index."""
    import hann_gb300 as hg
    import oracle

    oracle.build()
    oracle.set_tier(oracle.TIER_NEON)
    rng = np.random.default_rng(args.seed + 101)
    n, dim, nc, nqq, k = 20_000, 128, 64, 1000, 10
    cent = rng.normal(size=(nc, dim))
    x = (cent[rng.integers(0, nc, n)] + 0.3 * rng.normal(size=(n, dim))).astype(np.float32)
    qs = (cent[rng.integers(0, nc, nqq)] + 0.3 * rng.normal(size=(nqq, dim))).astype(np.float32)
    ids = np.arange(n, dtype=np.int64)
    cinit = rng.permutation(n)[:64]
    pinit = np.stack([rng.permutation(n)[:256] for _ in range(8)])
    reseed = rng.integers(0, n, 10000)
    cores = os.cpu_count() or 1
    gt, _ = oracle.brute_force_knn_fp64(qs, x, k, "euclidean", base_ids=ids)
    out = {"workload": f"{n} x {dim} Gaussian mixture (64 centres, sigma 0.3); coarse 64; 8 x 256 PQ; 10 "
                       f"k-means iterations from one seeded init; {nqq} queries; k {k}; nprobe 3"}
    idx = hg.New(dim, hg.WithCoarseK(64), hg.WithNumSubquantizers(8), hg.WithPQK(256), hg.WithKMeansIters(10))
    idx.BulkAddArrays(ids, x)
    torch.cuda.synchronize()
    t = time.perf_counter()
    idx.TrainSeeded(cinit, pinit, reseed)
    torch.cuda.synchronize()
    g_train = time.perf_counter() - t
    idx.SearchBatch(qs, k, mode=0)
    t = time.perf_counter()
    g_ids, g_d, g_n = idx.SearchBatch(qs, k, mode=0)
    g_batch = nqq / (time.perf_counter() - t)
    lat = []
    for i in range(nqq):
        t = time.perf_counter()
        idx.Search(qs[i], k)
        lat.append(time.perf_counter() - t)
    t = time.perf_counter()
    ora, info = oracle.train(ids, x, 64, 8, 256, 10, cinit, pinit, reseed, nthreads=cores)
    c_train = time.perf_counter() - t
    t = time.perf_counter()
    o_res = ora.search(qs, k, 3, nthreads=cores)
    c_batch = nqq / (time.perf_counter() - t)
    clat = []
    for i in range(nqq):
        t = time.perf_counter()
        ora.search(qs[i:i + 1], k, 3, nthreads=1)
        clat.append(time.perf_counter() - t)
    st = idx.export_state()
    g_asg = oracle.assign(x, st["coarse"], cores)
    gi = oracle.inertia_fp64(x, st["coarse"], g_asg)
    oi = oracle.inertia_fp64(x, ora.coarse, info["assign"])
    on_gpu_index = oracle_index_from_state(st).search(qs, k, 3, nthreads=cores)
    out["gpu"] = {"train_s": round(g_train, 4), "queries_per_s_batched": g_batch,
                  "p50_ms_one_query_per_call": 1e3 * float(np.percentile(lat, 50)),
                  "p99_ms_one_query_per_call": 1e3 * float(np.percentile(lat, 99)),
                  "recall_at_10_vs_fp64": recall_at(g_ids, gt), "coarse_inertia_fp64": gi}
    out["cpu_oracle"] = {"train_s": round(c_train, 3), "cores": cores, "queries_per_s_batched": c_batch,
                         "p50_ms_one_query_per_call": 1e3 * float(np.percentile(clat, 50)),
                         "p99_ms_one_query_per_call": 1e3 * float(np.percentile(clat, 99)),
                         "recall_at_10_vs_fp64": recall_at(o_res[0], gt), "coarse_inertia_fp64": oi,
                         "kind": "port (the reference's Train and Search restated in C, NEON order)"}
    out["inertia_rel_diff"] = abs(gi - oi) / oi
    out["search_parity_on_gpu_index"] = compare_results(g_ids, g_d, g_n, *on_gpu_index[:3])
    idx.close()
    log("config1", out)
    return out


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
        out[name] = {"train_s": round(el, 3), "s_per_iteration": round(el / iters, 4), "inertia_fp64": inertia,
                     "phases": idx.TrainPhases()}
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
                out["served_stream_1Mx128"] = []
                for rate in [float(r) for r in args.serve_rate.split(",") if r]:
                    try:
                        out["served_stream_1Mx128"].append(
                            serve_stream(args, idx, qs.cpu().numpy(), gt, nq_s, rate, n_ids=n,
                                         seconds=min(4.0, args.serve_seconds)))
                    except Exception as e:  # pragma: no cover
                        out["served_stream_1Mx128"].append({"offered_requests_per_s": rate, "error": str(e)})
                log("served 1Mx128", out["served_stream_1Mx128"])
            except Exception as e:  # pragma: no cover
                out["served_stream_1Mx128"] = {"error": str(e)}
        idx.close()
    a, b = states["tensor_core"], states["plain_fp32"]
    out["identical_index"] = bool(all(np.array_equal(a[key], b[key]) for key in ("coarse", "list_len", "ids",
                                                                                "codes")))
    if args.train_oracle_iters > 0 and not args.no_cpu_baseline:
        try:
            out["oracle_check"] = train_oracle_check(args, torch, dev, x, xh, k)
            log("train oracle check", out["oracle_check"])
        except Exception as e:  # pragma: no cover
            out["oracle_check"] = {"error": str(e)}
    return out


def train_oracle_check(args, torch, dev, x, xh, k):
    """Coarse k-means on the 1M x 128, k 4,096 shape from one seeded init,
    on the GPU (Train with that init) and in the oracle (runKMeans restated
    in C, all host cores), for args.train_oracle_iters iterations (fewer than
    the workload's 25: each oracle iteration is ~5e11 multiply-adds on the
    CPU). Reports both inertias (FP64, every point to its nearest centroid)
    and the CPU's seconds per iteration."""
    import hann_gb300 as hg
    import oracle

    oracle.build()
    oracle.set_tier(oracle.TIER_NEON)
    n, dim = xh.shape
    T = args.train_oracle_iters
    rng = np.random.default_rng(args.seed + 13)
    cinit = rng.permutation(n)[:k]
    pinit = np.stack([rng.permutation(n)[:256] for _ in range(16)])
    reseed = rng.integers(0, n, 100000)
    idx = hg.New(dim, hg.WithCoarseK(k), hg.WithNumSubquantizers(16), hg.WithPQK(256), hg.WithKMeansIters(T))
    idx.BulkAddArrays(np.arange(n, dtype=np.int64), xh)
    idx.TrainSeeded(cinit, pinit, reseed)
    g_cent = idx.export_state()["coarse"]
    idx.close()
    cores = os.cpu_count() or 1
    t = time.perf_counter()
    o_cent, _ = oracle.kmeans(xh, k, T, cinit, reseed, nthreads=cores)
    c_s = time.perf_counter() - t

    def inertia(cent):
        c = torch.from_numpy(np.ascontiguousarray(cent)).to(dev)
        cn = (c * c).sum(1)
        tot = 0.0
        for s0 in range(0, n, 1 << 16):
            xb = x[s0:s0 + (1 << 16)]
            a = torch.argmin(cn[None, :] - 2.0 * xb @ c.T, dim=1)
            d = xb.double() - c[a].double()
            tot += float((d * d).sum().item())
        return tot

    torch.backends.cuda.matmul.allow_tf32 = False
    gi, oi = inertia(g_cent), inertia(o_cent)
    return {"iterations": T, "gpu_inertia_fp64": gi, "oracle_inertia_fp64": oi, "rel_diff": abs(gi - oi) / oi,
            "cpu_s_per_iteration": c_s / T, "cores": cores,
            "what": "coarse k-means from the same seeded init and reseed stream, GPU Train vs the oracle's "
                    "runKMeans restatement; CPU seconds per iteration are the oracle's (assignment dominates)"}


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
    """DRAM bytes (read + write) of one scan stage (the scan kernel and its
    selection kernel) on this workload, from the 1-pass ncu capture kept in
    profiles/ (ncu cannot run inside the bench); None when the capture was of
    another workload."""
    path = os.path.join(HERE, "profiles", "scan_adc_kernel_10Mx96_dram.json")
    try:
        rec = json.load(open(path))
        if (rec["n"], rec["dim"], rec["nlist"], rec["M"], rec["nq"], rec["nprobe"], rec["k"]) != \
                (args.n, args.dim, args.nlist, args.m, args.nq, nprobe, args.k) or args.adc_tables != "fixed16":
            return None
        return float(rec["dram_bytes_read_per_launch"]) + float(rec["dram_bytes_write_per_launch"])
    except Exception:
        return None


def serve_schedule(args, rate, dur, nr, dim, n_ids, seed, id_base=50_000_000):
    """The served stream's arrival schedule, drawn before the clock starts:
    Poisson arrivals at `rate` requests/s for `dur` seconds; a search of
    1-512 queries (log-uniform) with k uniform in [1, 100] and nprobe
    log-uniform in [8, 256], or (1% each) a BulkAdd of 1,000 random unit
    vectors (ids from id_base up) or a BulkDelete of 100 random ids. Every
    fourth search with k >= 10 keeps its ids for the recall. Returns the
    request records of hann_serve_request and the arrays they point into."""
    import hann_gb300 as hg

    rng = np.random.default_rng(seed)
    n_req = int(rng.poisson(rate * dur))
    at = np.sort(rng.uniform(0.0, dur * 1000.0, n_req))
    u = rng.random(n_req)
    reqs = np.zeros(n_req, dtype=hg.Server.REQUEST_DTYPE)
    reqs["at_ms"] = at
    rows, add_ids, add_vecs, del_ids = [], [], [], []
    n_rows = n_add = n_del = n_out = 0
    next_id = id_base
    kept, searches = [], 0
    for i in range(n_req):
        if u[i] < 0.01:
            # random unit vectors: far from every query, so they do not
            # disturb the recall measured against the original ground truth
            chunk = rng.standard_normal((1000, dim)).astype(np.float32)
            chunk /= np.linalg.norm(chunk, axis=1, keepdims=True)
            add_vecs.append(chunk)
            add_ids.append(np.arange(next_id, next_id + 1000, dtype=np.int64))
            next_id += 1000
            reqs[i]["kind"], reqs[i]["first"], reqs[i]["count"] = 1, n_add, 1000
            n_add += 1000
        elif u[i] < 0.02:
            del_ids.append(rng.integers(0, n_ids, 100).astype(np.int64))
            reqs[i]["kind"], reqs[i]["first"], reqs[i]["count"] = 2, n_del, 100
            n_del += 100
        else:
            nq = int(np.exp(rng.uniform(0, np.log(512))))
            k = int(rng.integers(1, 101))
            npb = int(np.exp(rng.uniform(np.log(8), np.log(256))))
            r = rng.integers(0, nr, nq)
            rows.append(r)
            reqs[i]["kind"], reqs[i]["k"], reqs[i]["nprobe"] = 0, k, npb
            reqs[i]["first"], reqs[i]["count"] = n_rows, nq
            n_rows += nq
            reqs[i]["out_offset"] = -1
            if k >= 10:
                if searches % 4 == 0:
                    reqs[i]["out_offset"] = n_out
                    kept.append((i, r, k, n_out))
                    n_out += nq * k
                searches += 1
    cat = lambda xs, dt, shape: np.concatenate(xs) if xs else np.zeros(shape, dt)  # noqa: E731
    return (reqs, cat(rows, np.int64, (0,)), cat(add_ids, np.int64, (0,)), cat(add_vecs, np.float32, (0, dim)),
            cat(del_ids, np.int64, (0,)), kept, n_out)


_SERVE_NEXT_ID = [50_000_000]  # ids of the rows the served streams add, fresh in every phase


def serve_stream(args, idx, q_host, gt, nr, rate, n_ids=None, seconds=None):
    """The served stream (serve_schedule's requests) replayed by the
    library's native load generator (hann_serve_replay): the calling thread
    keeps to the arrival schedule natively and a native thread waits for
    every request, so the interpreter sets neither the arrivals nor the
    latencies. Reports p50/p99 latency (submit to result, the server's
    clock), queries/s, recall@10 over the kept searches, the relayout holds
    and how late the submissions were against the schedule."""
    import hann_gb300 as hg

    dur = seconds or args.serve_seconds
    reqs, rows, add_ids, add_vecs, del_ids, kept, n_out = serve_schedule(
        args, rate, dur, nr, q_host.shape[1], n_ids or args.n, args.seed + 7, _SERVE_NEXT_ID[0])
    _SERVE_NEXT_ID[0] += len(add_ids)
    srv = hg.Server(idx, slots=4, max_batch_queries=8192, max_k=100, max_nprobe=256, mode=1,
                    memory_budget=120 << 30, max_batch_probes=args.serve_batch_probes)
    try:
        lat, late, out = srv.replay(reqs, q_host, rows, add_ids, add_vecs, del_ids, n_out)
        st = srv.stats()
    finally:
        srv.stop()
    hits = tot = 0
    for i, r, k, off in kept:
        ids = out[off:off + len(r) * k].reshape(len(r), k)
        for j, row in enumerate(r):
            hits += len(set(ids[j, :10].tolist()) & set(gt[row].tolist()))
            tot += 10
    searches = reqs["kind"] == 0
    return {"requests": int(st["requests"]), "queries": int(st["queries"]), "batches": int(st["batches"]),
            "mutations": int(st["mutations"]), "p50_ms": st["p50_ms"], "p99_ms": st["p99_ms"],
            "search_p99_ms": round(float(np.percentile(lat[searches], 99)), 3) if searches.any() else None,
            "queries_per_s": st["queries_per_s"], "offered_requests_per_s": rate,
            "offered_queries_per_s": float(reqs["count"][searches].sum()) / dur,
            "recall_at_10_k_ge_10": hits / tot if tot else None,
            "peak_admitted_bytes": int(st["peak_admitted_bytes"]), "relayouts": int(st["relayouts"]),
            "submit_late_ms_p99": round(float(np.percentile(late, 99)), 3) if len(late) else None,
            "submit_late_ms_max": round(float(late.max()), 3) if len(late) else None,
            "mutation_ms_total": round(st["mutation_ms"], 1), "relayout_drain_ms_total": round(st["drain_ms"], 1),
            "relayout_ms_total": round(st["relayout_ms"], 1), "relayout_max_ms": round(st["relayout_max_ms"], 1),
            "stream": "Poisson arrivals; 1-512 queries/request log-uniform; k U[1,100]; nprobe log-U[8,256]; "
                      "BulkAdd 1000-vector chunks and BulkDeletes of 100 ids at 1% of the request rate each; "
                      "exact rerank; native load generator",
            "max_batch_probes": args.serve_batch_probes, "seconds": dur}


def workload_config(args, nprobe, mode):
    return {
        "workload": f"pqivf-search {args.n // 1_000_000}M x {args.dim} unit-norm Gaussian mixture "
                    f"({args.centers} centers, sigma {args.sigma}); coarse {args.nlist}; "
                    f"{args.m} x {args.pqk} PQ; {args.nq} queries; k {args.k}; nprobe {nprobe}; "
                    f"{'exact FP32 rerank of raw vectors' if mode == 1 else 'reference PQ distances'}",
        "n": args.n, "dim": args.dim, "nlist": args.nlist, "M": args.m, "pq_k": args.pqk, "nq": args.nq,
        "k": args.k, "nprobe": nprobe, "mode": "exact_rerank" if mode == 1 else "parity",
        "l2": f"inputs larger than L2 ({args.n * args.m / 1e6:.0f} MB of codes, {args.n * args.m / 1e6:.0f} MB "
              f"of scan codes + {args.n * 4 / 1e6:.0f} MB of terms + "
              f"{args.n * args.dim * 4 / 1e9:.2f} GB raw vectors), no flush",
        "adc_tables": args.adc_tables,
    }


if __name__ == "__main__":
    sys.exit(main())
