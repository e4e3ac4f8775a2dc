"""Benchmark: bases/s into the filtered k-mer graph on one GB300.

Workload (one step = one full graph build over one batch of reads):
  seeded synthetic genome of 5 Mbp (GC 50%), 2.5M reads x 100 bp sampled
  from both strands at 50x, 1% iid substitutions + 0.1% single-base indels,
  k=31, c=5 (uint64 keys, saturating uint8 multiplicities).
A step = one swg_graph_build_device call with the default algorithm (the
bucketed one for this workload: occurrence total, level-1 hash-partition
scatter of the k-mer occurrence records, level-2 bucket scatter, per-bucket
counting + cutoff in shared-memory tables, survivor gather), with the packed
reads resident in HBM. --algo direct selects the one-pass HBM-table build
(HyperLogLog sizing, table clear, K1 extract/count, K2 cutoff/compaction).
L2 is flushed (a 256 MiB write) before every timed step.

Prints ONE JSON line (rank 0). `e2e` repeats the measurement through the
C-ABI call on HOST (pinned) packed reads, with the host->device copy of the
reads and the device->host copy of the filtered graph inside the timed
region. `--impl reference` times the reference's CPU path instead.

Multi-GPU (torchrun): every rank builds its own replica of the workload
(independent samples, no data-path collective); value = all bases / max time.
"""
from __future__ import annotations

import argparse
import gc
import json
import os
import statistics
import subprocess
import sys
import threading
import time
from pathlib import Path

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT / "swap-assembler_gb300"))

METRIC = "bases/s into filtered k-mer graph on 1 GB300"
# The plain single-sample workloads (seeded synthetic reads with these shapes
# and error rates); the bench line is quoted on workload 2 by default.
CONFIGS = {
    1: (dict(seed=1, genome_len=1_000_000, gc=0.5, n_reads=300_000, read_len=100, sub_rate=0.005),
        21, 2, "plain single-sample build: 1 Mbp uniform genome, 300k x 100 bp reads at 30x from "
               "both strands, 0.5% subs, k=21, c=2"),
    2: (dict(seed=2, genome_len=5_000_000, gc=0.5, n_reads=2_500_000, read_len=100,
             sub_rate=0.01, indel_rate=0.001),
        31, 5, "plain single-sample build: 5 Mbp genome (GC 50%), 2.5M x 100 bp reads at 50x "
               "from both strands, 1% subs + 0.1% indels, k=31, c=5"),
    3: (dict(seed=3, genome_len=100_000_000, gc=0.5, repeat_frac=0.05, tandem_frac=0.02,
             n_reads=20_000_000, read_len=150, sub_rate=0.005),
        31, 3, "plain single-sample build, skewed: 100 Mbp genome with 5% repeat families "
               "(1-5 kbp units, 2-200 copies, 1% divergence) + 2% tandem repeats (2-6 bp units), "
               "20M x 150 bp reads at 30x, 0.5% subs, k=31, c=3"),
}
WORKLOAD, K, CUTOFF, DESC = CONFIGS[2]
L2_FLUSH_BYTES = 256 << 20


def parse_args():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--no-probe", action="store_true", help="skip the random-access probe")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-batch", action="store_true", help="skip the batched-samples measurement")
    ap.add_argument("--no-serve", action="store_true", help="skip the served-requests measurement")
    ap.add_argument("--no-merge", action="store_true", help="skip the merge-stage measurement")
    ap.add_argument("--algo", default="default", choices=["default", "direct", "partitioned", "bucketed"])
    ap.add_argument("--order", default="input", choices=["input", "minimizer"],
                    help="read order of the direct algorithm")
    ap.add_argument("--reads", type=int, default=0,
                    help="smaller case for profiling: this many reads, genome scaled to keep the coverage")
    ap.add_argument("--config", type=int, default=2, choices=sorted(CONFIGS),
                    help="plain workload: 1 = 1 Mbp/30x/k21 c2, 2 = 5 Mbp/50x/k31 c5 (default), "
                         "3 = 100 Mbp with repeats/30x/150 bp/k31 c3")
    args = ap.parse_args()
    global WORKLOAD, K, CUTOFF, DESC
    WORKLOAD, K, CUTOFF, DESC = CONFIGS[args.config]
    return args


def config_dict() -> dict:
    """The workload, the same for both arms (what each arm runs on it is in
    its "arm" key)."""
    return {"workload": DESC, "genome_bp": WORKLOAD["genome_len"], "reads": WORKLOAD["n_reads"],
            "read_len": WORKLOAD["read_len"], "k": K, "c": CUTOFF,
            "l2": "flushed (256 MiB write) before every GPU step"}


class ClockSampler:
    """nvidia-smi clocks sampled every 200 ms while the timed region runs."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.gpu = gpu_index
        self.proc = None
        self.lines: list[str] = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.gpu), "--query-gpu=" + self.FIELDS,
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except OSError:
            self.proc = None
        time.sleep(0.3)
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *exc):
        if self.proc:
            time.sleep(0.25)
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self) -> dict | None:
        rows = []
        for l in self.lines:
            parts = [p.strip() for p in l.split(",")]
            if len(parts) < 9:
                continue
            try:
                rows.append((float(parts[1]), float(parts[2]), parts[5:9]))
            except ValueError:
                continue
        if not rows:
            return None
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for _, _, r in rows for i in range(4) if r[i] == "Active"})
        return {"sm_mhz": statistics.median(r[0] for r in rows), "sm_max_mhz": max(r[1] for r in rows),
                "reasons": reasons, "samples": len(rows)}


def measured_peaks() -> dict:
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        try:
            return json.loads(p.read_text())
        except ValueError:
            pass
    return {}


def traffic_per_occ(kernel: str) -> tuple[float | None, str | None]:
    """DRAM bytes (read + write) per k-mer occurrence of one kernel, from an
    ncu capture summarised under profiles/ (scaled to a full launch by the
    occurrences it processes)."""
    p = ROOT / "profiles" / ("%s_ncu.json" % kernel)
    if not p.exists():
        return None, None
    d = json.loads(p.read_text())
    return d.get("dram_bytes_per_occurrence"), d.get("source")


def cpu_baseline(text: bytes, n_bases: int, budget_s: float = 20.0) -> dict:
    """The oracle port timed on this host's cores on a bounded prefix sample."""
    sys.path.insert(0, str(ROOT / "oracle"))
    import oracle
    threads = oracle.cores()
    # calibrate on ~2% of the reads, then size the sample for about budget_s
    cut = lambda frac: text[: text.index(b"\n>", int(len(text) * frac)) + 1]
    t0 = time.perf_counter()
    small = cut(0.02)
    oracle.records(small, K, CUTOFF, threads)
    dt = max(time.perf_counter() - t0, 1e-3)
    frac = min(1.0, 0.02 * budget_s / dt / 2)
    sample = text if frac >= 1.0 else cut(frac)
    nb = oracle.parse(sample, K)["n_bases"]
    t0 = time.perf_counter()
    oracle.records(sample, K, CUTOFF, threads)
    dt = time.perf_counter() - t0
    return {"value": nb / dt, "unit": "bases/s", "cores": threads, "kind": "port",
            "sample": "first %d of %d bases (framing + count + cutoff, sorted records), %.1f s"
                      % (nb, n_bases, dt)}


# Random accesses per k-molecule the GPU merge makes (merge.cu): index insert
# 1, one neighbour lookup per arc (about 2), the two neighbours' flags 2, per
# walk state one 16-byte successor load and one label store (4), the chain
# entry 1 and the two arc-string bases 2.
MERGE_RANDOM_PER_NODE = 12


def merge_metrics(g, survivors: int, steps: int, warmup: int) -> dict:
    """swg_graph_merge on the graph just built (device time from the library's
    CUDA events, which cover its host synchronisations too)."""
    for _ in range(max(warmup, 3)):
        g.merge()
    ms = []
    for _ in range(steps):
        g.merge()
        ms.append(g.merge_info()["ms"])
    info = g.merge_info()
    m = statistics.median(ms)
    # the reference's rank-0 sequence on the merged graph: tip pass,
    # simplify, low-coverage pass, simplify (wall time of each call: the
    # kernels, the text rewrite and its host synchronisations)
    t0 = time.perf_counter()
    tips = g.remove_tips()
    t1 = time.perf_counter()
    s1 = g.simplify()
    t2 = time.perf_counter()
    cut = g.remove_low_coverage()
    t3 = time.perf_counter()
    s2 = g.simplify()
    t4 = time.perf_counter()
    return {"what": "merging of semi-extended k-molecules (simplifyDistNodeGraph) over the built graph, "
                    "result = the -d file's text on the device",
            "ms": m, "ms_all": ms, "k_molecules": survivors, "k_molecules_per_s": survivors / (m * 1e-3),
            "nodes_left": info["nodes"], "chains": info["chains"], "cycles": info["cycles"],
            "text_bytes": info["text_bytes"], "launches": info["launches"],
            "random_accesses_per_k_molecule": MERGE_RANDOM_PER_NODE,
            "tips": {"wall_ms": (t1 - t0) * 1e3, "removed": tips},
            "simplify_after_tips": {"wall_ms": (t2 - t1) * 1e3, "merged": s1},
            "low_coverage": {"wall_ms": (t3 - t2) * 1e3, "arcs_cut": cut},
            "simplify_after_low_coverage": {"wall_ms": (t4 - t3) * 1e3, "merged": s2,
                                            "nodes_left": g.merge_info()["nodes"]}}


MERGE_CPU_MAX = 8_000_000  # k-molecules: about 40 s for the one-thread restatement


def merge_cpu_baseline(g, k: int) -> dict:
    """The CPU restatement of the merge (one thread) on the same k-molecules.
    The merge needs the whole graph (chains run through it), so a graph past
    MERGE_CPU_MAX k-molecules is not timed: it would take minutes."""
    n = g.size()
    if n > MERGE_CPU_MAX:
        return {"value": None, "unit": "k-molecules/s", "cores": 1, "kind": "port",
                "sample": "not run: %d k-molecules, past the %d that finish in about 40 s"
                          % (n, MERGE_CPU_MAX)}
    sys.path.insert(0, str(ROOT / "oracle"))
    import oracle
    keys, mult = g.copy_out(sorted=True)
    t0 = time.perf_counter()
    order = oracle.merge_tree_order(keys, mult.reshape(-1, 8), k)
    oracle.merge_text(keys, mult.reshape(-1, 8), k, order=order)
    dt = time.perf_counter() - t0
    return {"value": keys.size / dt, "unit": "k-molecules/s", "cores": 1, "kind": "port",
            "sample": "the whole graph: %d k-molecules (visiting order + merge + text), %.1f s"
                      % (keys.size, dt)}


def batched_samples(n: int = 256, seed: int = 4) -> list[dict]:
    """The batched workload: genome sizes log-uniform 50 kbp-2 Mbp, read length
    from {75, 100, 150, 250}, coverage uniform 10-60x, substitutions uniform
    0.1-1%, k=27, c=3 for every sample."""
    import swapgb
    return swapgb.batch_workload_specs(n, seed)


def batched_metrics(stream_ptr: int, repeats: int = 3) -> dict:
    """Samples/s of one batched build over all samples vs one plain build per
    sample, both from host packed reads to device-resident results."""
    import numpy as np
    import torch
    import swapgb
    specs = batched_samples()

    class PinnedReads:
        """A sample's packed reads staged in pinned host memory (both arms read it)."""

        def __init__(self, r):
            self._t = [torch.from_numpy(a.copy()).pin_memory()
                       for a in (r.packed.view(np.int32), r.off.view(np.int64), r.len.view(np.int32))]
            self.packed = self._t[0].numpy().view(np.uint32)
            self.off = self._t[1].numpy().view(np.uint64)
            self.len = self._t[2].numpy().view(np.uint32)
            self.n_words, self.n_reads, self.n_bases = r.n_words, r.n_reads, r.n_bases

    reads = [PinnedReads(swapgb.reads_from_fasta(swapgb.synth_fasta(**p), 27)) for p in specs]
    bases = sum(r.n_bases for r in reads)
    opts = swapgb.Opts(k=27, cutoff=3, stream=stream_ptr)
    plain, batch = swapgb.Graph(), swapgb.Graph()
    samples = [(r, 27, 3) for r in reads]
    batch.build_batch(opts, samples)  # warm-up (allocations)
    for r in reads:
        plain.build_reads(opts, r)
    torch.cuda.synchronize()
    t_plain, t_batch, dev_plain, dev_batch = [], [], [], []
    for _ in range(repeats):
        t0 = time.perf_counter()
        dp = 0.0
        for r in reads:
            plain.build_reads(opts, r)
            dp += plain.info()["ms"][4]
        torch.cuda.synchronize()
        t_plain.append(time.perf_counter() - t0)
        dev_plain.append(dp)
        t0 = time.perf_counter()
        batch.build_batch(opts, samples)
        torch.cuda.synchronize()
        t_batch.append(time.perf_counter() - t0)
        dev_batch.append(batch.info()["ms"][4])
    # every sample of the batch against its own plain build (outside the timing)
    same = 0
    for i, r in enumerate(reads):
        plain.build_reads(opts, r)
        kp, mp = plain.copy_out(sorted=True)
        kb, mb = batch.batch_copy_out(i)
        same += bool(np.array_equal(kp, kb) and np.array_equal(mp, mb))
    # the autotuner over the bucketed knobs, on two samples of each read length
    # built as one sample with the batch's k (its choice then runs the batch)
    pick = []
    for L in (75, 100, 150, 250):
        pick += [i for i, p in enumerate(specs) if p["read_len"] == L][:2]
    words = np.concatenate([reads[i].packed for i in pick])
    shift = np.cumsum([0] + [reads[i].n_words * 16 for i in pick[:-1]]).astype(np.uint64)
    offs = np.concatenate([reads[i].off + shift[j] for j, i in enumerate(pick)])
    lens = np.concatenate([reads[i].len for i in pick])
    d_w = torch.from_numpy(words.view(np.int32)).cuda()
    d_o = torch.from_numpy(offs.view(np.int64)).cuda()
    d_l = torch.from_numpy(lens.view(np.int32)).cuda()
    import tempfile
    with tempfile.TemporaryDirectory() as td:
        best = swapgb.autotune(swapgb.Opts(k=27, cutoff=3, stream=stream_ptr), d_w.data_ptr(), d_w.numel(),
                               d_o.data_ptr(), d_l.data_ptr(), d_o.numel(), 150, os.path.join(td, "tune.jsonl"))
    tuned = swapgb.Opts(k=27, cutoff=3, stream=stream_ptr)
    if best["algorithm"] == swapgb.ALGO_BUCKETED:
        tuned.bucket_records, tuned.part_bits = best["bucket_records"], best["part_bits"]
        tuned.scatter_shape = best["scatter_shape"]
    batch.build_batch(tuned, samples)
    torch.cuda.synchronize()
    t_tuned = []
    for _ in range(repeats):
        t0 = time.perf_counter()
        batch.build_batch(tuned, samples)
        torch.cuda.synchronize()
        t_tuned.append(time.perf_counter() - t0)
    tuned_same = 0
    for i in range(len(reads)):
        kb, mb = batch.batch_copy_out(i)
        plain.build_reads(opts, reads[i])
        kp, mp = plain.copy_out(sorted=True)
        tuned_same += bool(np.array_equal(kp, kb) and np.array_equal(mp, mb))
    tp, tb = min(t_plain), min(t_batch)
    return {"workload": "256 samples, genome log-uniform 50 kbp-2 Mbp, reads 75/100/150/250 bp, "
                        "10-60x, 0.1-1% subs, k=27 c=3 (seeded synthetic)",
            "samples": len(reads), "bases": bases,
            "plain_s": tp, "batched_s": tb,
            "plain_samples_per_s": len(reads) / tp, "batched_samples_per_s": len(reads) / tb,
            "batched_bases_per_s": bases / tb, "speedup": tp / tb,
            "device_ms_plain_sum": min(dev_plain), "device_ms_batched": min(dev_batch),
            "batched_algorithm": {1: "direct", 2: "partitioned", 3: "bucketed"}[batch.info()["algorithm"]],
            "samples_identical": "%d/%d" % (same, len(reads)),
            "autotune": {"picked": best, "on": "2 samples of each read length built as one sample (k=27, c=3)",
                         "batched_s": min(t_tuned), "batched_samples_per_s": len(reads) / min(t_tuned),
                         "speedup": tp / min(t_tuned),
                         "samples_identical": "%d/%d" % (tuned_same, len(reads))},
            "identical_means": "the sample's sorted k-molecules and 8 multiplicities equal its own plain "
                               "build's, bit for bit",
            "path": "pinned host packed reads -> device-resident graphs; plain = swg_graph_build "
                    "per sample, batched = one swg_batch_build"}


SERVED_RATES = (50.0, 200.0, 800.0, 3200.0)  # req/s of the served sweep
SERVED_REQUESTS = 800                         # at most this many requests per rate


def served_metrics(stream_ptr: int) -> dict:
    """Poisson request streams through the request server, one per rate of
    SERVED_RATES (10 s, or SERVED_REQUESTS requests at the higher rates).
    Request sizes follow the batched workload's per-sample distribution, plus
    2% large requests (10 Mbp genome, 40x, 150 bp reads); k from
    {21, 25, 27, 31} and c from {2, 3, 5} per request; 150 GiB admission
    budget. A pool of distinct request inputs is generated once and drawn
    from. Every result is fetched and its SHA-256 (sorted records) compared,
    after the stream, with a plain build of the same input, k and c; the
    plain builds' wall times give the plain form's samples/s for the mix."""
    import hashlib
    import random
    import threading
    import numpy as np
    import torch
    import swapgb
    specs = batched_samples(n=40, seed=5)
    pool = [swapgb.reads_from_fasta(swapgb.synth_fasta(**p), 21) for p in specs]
    large = swapgb.reads_from_fasta(swapgb.synth_fasta(seed=77, genome_len=10_000_000,
                                                       n_reads=2_666_667, read_len=150,
                                                       sub_rate=0.005), 21)
    inputs = pool + [large]
    digest = lambda k, m: hashlib.sha256(k.tobytes() + m.tobytes()).hexdigest()

    def one_rate(rate: float, seed: int) -> tuple[dict, list]:
        rng = random.Random(seed)
        srv = swapgb.Server(memory_budget=150 << 30, workers=2)
        for r in (pool[0], large):  # warm-up: one request of each kind
            t = srv.submit(r, 27, 3)
            srv.wait(t, 120.0)
            srv.release(t)
        base = srv.stats()
        duration = min(10.0, SERVED_REQUESTS / rate)
        tickets, reqs, t_sub = [], [], []  # reqs: (input index, k, c); submit times (s)
        lock = threading.Lock()
        done = threading.Event()
        got = {}  # ticket -> (latency s, keys, multiplicities), checked after the stream

        def collector():
            i = 0
            while True:
                with lock:
                    t = tickets[i] if i < len(tickets) else None
                if t is None:
                    if done.is_set():
                        with lock:
                            if i >= len(tickets):
                                return
                        continue
                    time.sleep(0.0005)
                    continue
                srv.wait(t, 300.0)
                lat = srv.poll(t)[1]  # completion - submission, taken by the server
                k, m = srv.fetch(t, sorted=False)  # a copy only; sorted and hashed after the stream
                got[t] = (lat, k, m)
                i += 1

        th = threading.Thread(target=collector)
        th.start()
        t0 = time.perf_counter()
        t_next = 0.0
        while t_next < duration:
            now = time.perf_counter() - t0
            if now < t_next:
                time.sleep(t_next - now)
            j = len(inputs) - 1 if rng.random() < 0.02 else rng.randrange(len(pool))
            k, c = rng.choice([21, 25, 27, 31]), rng.choice([2, 3, 5])
            ts = time.perf_counter() - t0
            t = srv.submit(inputs[j], k, c)
            with lock:
                tickets.append(t)
                reqs.append((j, k, c))
                t_sub.append(ts)
            t_next += rng.expovariate(rate)
        done.set()
        th.join()
        st = srv.stats()
        srv.close()
        lats = sorted(got[t][0] for t in tickets)
        q = lambda f: lats[min(len(lats) - 1, int(f * len(lats)))]
        # the stream's span: first submission to the last result resident
        span = max(t_sub[i] + got[t][0] for i, t in enumerate(tickets)) - t_sub[0]
        n_batches = st["batches"] - base["batches"]
        bases = sum(inputs[j].n_bases for j, _, _ in reqs)
        row = {"rate_req_per_s": rate, "seconds": duration, "requests": len(tickets),
               "large_requests": sum(j == len(inputs) - 1 for j, _, _ in reqs),
               "p50_ms": 1e3 * q(0.50), "p99_ms": 1e3 * q(0.99), "max_ms": 1e3 * lats[-1],
               "span_s": span, "aggregate_samples_per_s": len(tickets) / span,
               "aggregate_bases_per_s": bases / span, "offered_bases_per_s": bases / duration,
               "batches": n_batches, "mean_batch_requests": len(tickets) / max(n_batches, 1),
               "max_batch_requests": st["max_batch_requests"]}
        from concurrent.futures import ThreadPoolExecutor

        def check(i):
            _, kk, mm = got[tickets[i]]
            o = np.argsort(kk, kind="stable")
            return reqs[i], digest(kk[o], mm[o])
        with ThreadPoolExecutor(max_workers=min(16, os.cpu_count() or 1)) as ex:
            checks = list(ex.map(check, range(len(tickets))))
        got.clear()
        return row, checks

    rows, checks = [], []
    for i, rate in enumerate(SERVED_RATES):
        row, chk = one_rate(rate, seed=5 + i)
        rows.append(row)
        checks.append(chk)
    # every fetched result against a plain build of the same request
    g = swapgb.Graph()
    want, plain_s = {}, {}
    for combo in sorted({c for chk in checks for c, _ in chk}):
        j, k, c = combo
        opts = swapgb.Opts(k=k, cutoff=c, stream=stream_ptr)
        g.build_reads(opts, inputs[j])  # warm (allocations), then timed
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        g.build_reads(opts, inputs[j])
        torch.cuda.synchronize()
        plain_s[combo] = time.perf_counter() - t0
        want[combo] = digest(*g.copy_out(sorted=True))
    for row, chk in zip(rows, checks):
        row["results_identical"] = "%d/%d" % (sum(want[c] == d for c, d in chk), len(chk))
        row["plain_samples_per_s"] = len(chk) / sum(plain_s[c] for c, _ in chk)
    return {"workload": "Poisson request streams at %s req/s (10 s or %d requests each); sizes from the "
                        "batched workload's per-sample distribution + 2%% large (10 Mbp, 40x, 150 bp); k in "
                        "{21,25,27,31}, c in {2,3,5}; 150 GiB budget; 2 workers"
                        % ("/".join("%g" % r for r in SERVED_RATES), SERVED_REQUESTS),
            "latency": "submit (including the server's copy of the reads) to the result resident on the "
                       "device",
            "aggregate_means": "requests (bases) over the span from the first submission to the last "
                               "result resident on the device",
            "results_identical_means": "SHA-256 of the fetched sorted records equals a plain build's of the "
                                       "same input, k and c",
            "plain_samples_per_s_means": "the same requests built one by one with swg_graph_build from host "
                                         "packed reads (wall time per build, result on the device)",
            "sweep": rows}


def run_reference_arm(args) -> int:
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return 0
    import swapgb
    sys.path.insert(0, str(ROOT / "oracle"))
    import oracle
    text = swapgb.synth_fasta(**WORKLOAD)
    kind = "port"
    threads = oracle.cores()
    # every step is the whole workload: the FASTA text in host memory framed,
    # counted and cut off (about 3 s on 16 cores for workload 2)
    nb = oracle.parse(text, K)["n_bases"]
    for _ in range(max(args.warmup, 0)):
        oracle.records(text, K, CUTOFF, threads)
    times = []
    for _ in range(args.steps):
        t0 = time.perf_counter()
        oracle.records(text, K, CUTOFF, threads)
        times.append(time.perf_counter() - t0)
    ms = 1e3 * statistics.mean(times)
    value = nb / (ms * 1e-3)
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": "bases/s",
        "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "u64",
        "data": "synthetic (seeded generator, no dataset)", "config": config_dict(),
        "arm": {"runs": "the reference's algorithm restated in C (oracle/kmer_oracle.c), one thread "
                        "per MPI rank of the reference's scheme, on the host cores",
                "inputs": "the workload's FASTA text in host memory"},
        "cpu_baseline": {"value": value, "unit": "bases/s", "cores": threads, "kind": kind,
                         "sample": "the whole workload every step: %d bases (framing + count + "
                                   "cutoff, sorted records)" % nb},
        "e2e": {"value": value, "unit": "bases/s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line))
    return 0


def max_over_ranks(x: float, world: int, device=None) -> float:
    """The slowest rank's value (timings are reported as the max over ranks)."""
    if world <= 1:
        return x
    import torch
    import torch.distributed as dist
    t = torch.tensor([x], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def aggregate_value(bases_per_rank: int, world: int, ms_slowest: float) -> float:
    """Whole-job bases/s: every rank builds its own replica (weak scaling)."""
    return world * bases_per_rank / (ms_slowest * 1e-3)


def main() -> int:
    args = parse_args()
    if args.impl == "reference":
        return run_reference_arm(args)
    import numpy as np
    import torch
    import torch.distributed as dist

    import swapgb

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        dist.init_process_group("nccl")
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)

    work = dict(WORKLOAD)
    if args.reads:
        work["genome_len"] = max(10_000, WORKLOAD["genome_len"] * args.reads // WORKLOAD["n_reads"])
        work["n_reads"] = args.reads
    text = swapgb.synth_fasta(**work)
    reads = swapgb.reads_from_fasta(text, K)
    n_bases = reads.n_bases
    n_occ = int((reads.len.astype(np.int64) - K + 1).clip(min=0).sum())
    stream = torch.cuda.current_stream(dev)
    algo = {"default": swapgb.ALGO_DEFAULT, "direct": swapgb.ALGO_DIRECT,
            "partitioned": swapgb.ALGO_PARTITIONED, "bucketed": swapgb.ALGO_BUCKETED}[args.algo]
    order = swapgb.ORDER_MINIMIZER if args.order == "minimizer" else swapgb.ORDER_INPUT
    opts = swapgb.Opts(k=K, cutoff=CUTOFF, stream=stream.cuda_stream, algorithm=algo,
                       read_order=order)

    d_packed = torch.from_numpy(reads.packed.view(np.int32).copy()).to(dev)
    d_off = torch.from_numpy(reads.off.view(np.int64).copy()).to(dev)
    d_len = torch.from_numpy(reads.len.view(np.int32).copy()).to(dev)
    flush = torch.empty(L2_FLUSH_BYTES // 4, dtype=torch.int32, device=dev)
    g = swapgb.Graph()

    def step():
        g.build_device(opts, d_packed.data_ptr(), d_packed.numel(), d_off.data_ptr(),
                       d_len.data_ptr(), d_off.numel())

    for _ in range(max(args.warmup, 3)):
        flush.fill_(1)
        step()
    torch.cuda.synchronize()
    if world > 1:
        dist.barrier()
    evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
           for _ in range(args.steps)]
    phase_ms, launches = [], 0
    gc.collect()
    gc.disable()  # no collector pause inside the timed steps
    with ClockSampler(local) as clocks:
        torch.cuda.synchronize()
        t_wall0 = time.perf_counter()
        for i in range(args.steps):
            flush.fill_(i)
            evs[i][0].record(stream)
            step()
            evs[i][1].record(stream)
            ms, nl = g.timings()
            phase_ms.append(ms)
            launches += nl
        torch.cuda.synchronize()
        t_wall = time.perf_counter() - t_wall0
    gc.enable()
    step_ms = [a.elapsed_time(b) for a, b in evs]
    ms_per_step = max_over_ranks(statistics.mean(step_ms), world, dev)
    value = aggregate_value(n_bases, world, ms_per_step)
    survivors, distinct = g.size(), g.distinct()
    merge = None
    if rank == 0 and not args.no_merge:
        merge = merge_metrics(g, survivors, args.steps, args.warmup)

    # ---- end to end through the C ABI on pinned host buffers ----
    lib = swapgb.lib()
    h_keys = torch.empty(max(survivors, 1) + (1 << 20), dtype=torch.int64).pin_memory()
    h_mult = torch.empty_like(h_keys)
    g2 = swapgb.Graph()

    def copy_out_e2e() -> int:
        n = swapgb.C.c_uint64()
        swapgb._check(lib.swg_graph_copy_out(g2._h, h_keys.data_ptr(), h_mult.data_ptr(),
                                             h_keys.numel(), 0, swapgb.C.byref(n)), "copy_out")
        return n.value

    # (1) the FASTA text as a user has it: copied to the device, framed and
    # packed there, built, filtered graph copied back
    h_text = torch.from_numpy(np.frombuffer(text, dtype=np.uint8).copy()).pin_memory()

    def e2e_fasta() -> int:
        # one call: built from the text, survivors written into the pinned
        # host arrays while the buckets are counted
        n = swapgb.C.c_uint64()
        swapgb._check(lib.swg_graph_build_fasta_to_host(g2._h, swapgb.C.byref(opts), h_text.data_ptr(),
                                                        h_text.numel(), h_keys.data_ptr(), h_mult.data_ptr(),
                                                        h_keys.numel(), swapgb.C.byref(n)),
                      "swg_graph_build_fasta_to_host")
        return n.value

    def e2e_fasta_two_calls() -> int:
        swapgb._check(lib.swg_graph_build_fasta(g2._h, swapgb.C.byref(opts), h_text.data_ptr(),
                                                h_text.numel()), "swg_graph_build_fasta")
        return copy_out_e2e()

    # (2) host packed reads (swg_graph_build)
    h_packed = torch.from_numpy(reads.packed.view(np.int32).copy()).pin_memory()
    h_off = torch.from_numpy(reads.off.view(np.int64).copy()).pin_memory()
    h_len = torch.from_numpy(reads.len.view(np.int32).copy()).pin_memory()

    def e2e_packed() -> int:
        swapgb._check(lib.swg_graph_build(g2._h, swapgb.C.byref(opts), h_packed.data_ptr(),
                                          h_packed.numel(), h_off.data_ptr(), h_len.data_ptr(),
                                          h_off.numel()), "swg_graph_build")
        return copy_out_e2e()

    device_ms_steps = []  # the build's own event-timed total per timed step

    def timed(fn) -> tuple[float, int, list[float]]:
        for _ in range(2):
            fn()
        torch.cuda.synchronize()
        ts = []
        device_ms_steps.clear()
        gc.disable()  # no collector pause inside a timed step
        try:
            for _ in range(max(3, min(args.steps, 10))):
                t0 = time.perf_counter()
                n = fn()
                ts.append(time.perf_counter() - t0)
                device_ms_steps.append([round(x, 3) for x in g2.timings()[0]] + [g2.info()["estimate"]])
        finally:
            gc.enable()
        return max_over_ranks(statistics.mean(ts), world, dev), n, [round(t * 1e3, 3) for t in ts]

    e2e_s, n_e2e, e2e_steps = timed(e2e_fasta)
    e2e_build_ms_steps = list(device_ms_steps)
    e2e2_s, _, e2e2_steps = timed(e2e_fasta_two_calls)
    # where one end-to-end step goes: the build's event phases (the streamed
    # build's level-1 phase holds the upload and the framing of the pieces),
    # then the result copy alone
    e2e_fasta_two_calls()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    swapgb._check(lib.swg_graph_build_fasta(g2._h, swapgb.C.byref(opts), h_text.data_ptr(),
                                            h_text.numel()), "swg_graph_build_fasta")
    t1 = time.perf_counter()
    copy_out_e2e()
    t2 = time.perf_counter()
    e2e_phases = {"build_wall_ms": 1e3 * (t1 - t0), "copy_out_wall_ms": 1e3 * (t2 - t1),
                  "build_phase_ms": dict(zip(("setup", "level1_with_upload_and_framing", "level2",
                                              "bucket_count", "total"), g2.timings()[0]))}
    e2e_p_s, _, e2e_p_steps = timed(e2e_packed)

    # the documented drop-in from a FASTA file on local disk,
    # page cache warm: device framing (swg_graph_build_fasta_file) against host
    # framing (swg_reads_from_fasta_file + swg_graph_build), result on the device
    dropin = None
    if rank == 0 and not args.reads:
        import tempfile
        with tempfile.TemporaryDirectory() as td:
            fa = os.path.join(td, "reads.fa")
            with open(fa, "wb") as f:
                f.write(text)
            g3 = swapgb.Graph()

            def file_device():
                g3.build_fasta_file(opts, fa)
                torch.cuda.synchronize()

            def file_host():
                r = swapgb.reads_from_fasta_file(fa, K)
                g3.build_reads(opts, r)
                torch.cuda.synchronize()

            def wall(fn, n=3):
                fn()
                ts = []
                for _ in range(n):
                    t0 = time.perf_counter()
                    fn()
                    ts.append(time.perf_counter() - t0)
                return 1e3 * statistics.median(ts)
            dropin = {"what": "one build from the FASTA file (page cache warm) to the filtered graph on the device",
                      "file_device_framing_ms": wall(file_device), "file_host_framing_ms": wall(file_host),
                      "file_bytes": len(text)}
            g3.close()
    h2d = h_text.numel()
    h2d_p = h_packed.numel() * 4 + h_off.numel() * 8 + h_len.numel() * 4
    d2h = n_e2e * 16

    # ---- rooflines ----
    peaks = measured_peaks()
    hbm = peaks.get("hbm_gbs")
    peak_src = "of measured" if hbm else "of fallback"
    hbm = hbm or 6800.0
    info = g.info()
    used = info["algorithm"]  # what the default resolved to
    mean_ms = [statistics.mean(m[i] for m in phase_ms) for i in range(5)]
    n_with_occ = int((reads.len >= K).sum())
    kfile = None
    if used == swapgb.ALGO_DIRECT:
        kname, k_ms, kfile = "k_count", mean_ms[2], "k_count"
        algo_bytes = n_occ * 64 + n_bases / 4 + reads.n_reads * 12
        model = ("64 B per k-mer occurrence (one 32 B sector of the hash-table entry read + "
                 "written back) + 0.25 B per base + 12 B per read")
    elif used == swapgb.ALGO_BUCKETED:
        # the longer of the two single-kernel phases, each timed by events
        # around that kernel's launch on the build stream
        if mean_ms[1] >= mean_ms[3]:
            kname, k_ms, kfile = "k_p1_scatter", mean_ms[1], "k_p1_scatter"
            algo_bytes = n_bases / 4 + reads.n_reads * 12 + n_occ * 8
            model = ("packed reads in (0.25 B per base + 12 B per read), one 8 B record per "
                     "k-mer occurrence out")
        else:
            # the tier-1 configuration the build chose (2048-entry tables for
            # small buckets); the tier-2 recount is part of the same phase
            kname = "k_bucket_count_small" if info.get("bucket_table") == 2048 else "k_bucket_count"
            k_ms, kfile = mean_ms[3], kname
            algo_bytes = n_occ * 8 + survivors * 16
            model = "one 8 B record per k-mer occurrence in, 16 B per surviving k-molecule staged"
    else:
        # the whole partitioned build: every kernel, DRAM bytes it cannot avoid
        kname, k_ms = "partitioned build (all kernels)", mean_ms[4]
        algo_bytes = (n_occ * 16 + 2 * (n_bases / 4 + reads.n_reads * 12) + survivors * 16)
        model = ("8 B record written + read per k-mer occurrence, packed input read twice "
                 "(0.25 B/base + 12 B/read each), 16 B per surviving k-molecule written; "
                 "partition slices stay in L2")
    achieved = algo_bytes / (k_ms * 1e-3) / 1e9
    tpo, tsrc = traffic_per_occ(kfile) if kfile else (None, None)
    roofline = {"kernel": kname, "bound": "hbm", "achieved": achieved, "peak": hbm,
                "unit": "GB/s", "frac": achieved / hbm, "peak_source": peak_src,
                "traffic": (tpo * n_occ) if tpo else None, "traffic_source": tsrc,
                "algorithmic_bytes": algo_bytes, "bytes_model": model, "kernel_ms": k_ms}
    if kname.startswith("k_bucket_count") and not args.no_probe:
        # the kernel's own ceiling is on chip: one 64-bit shared CAS per record
        # (a lower bound: linear probing adds some) and one 32-bit shared add
        # per arc, at the rates this GPU's shared-memory atomics reach
        r_add = swapgb.probe_shared_atomics("add_u32", 1 << 31, stream.cuda_stream)
        r_cas = swapgb.probe_shared_atomics("cas_u64", 1 << 30, stream.cuda_stream)
        n_arcs = 2 * n_occ - 2 * n_with_occ
        floor_ms = 1e3 * (n_occ / r_cas + n_arcs / r_add)
        roofline["on_chip"] = {"bound": "shared-memory atomics", "floor_ms": floor_ms,
                               "frac": floor_ms / k_ms, "cas64_lane_ops_per_s": r_cas,
                               "add32_lane_ops_per_s": r_add, "cas_per_build": n_occ,
                               "adds_per_build": n_arcs,
                               "model": "one 64-bit shared atomicCAS per record + one 32-bit shared "
                                        "atomicAdd per arc, at the rates swg_probe_shared_atomics "
                                        "measures in the same table layout (this run)"}
    atomic = None
    if not args.no_probe and rank == 0:
        table_bytes = 16 << 30
        r_red = swapgb.probe_random_access("red_add_u32", table_bytes, 1 << 31, stream.cuda_stream)
        r_pat = swapgb.probe_random_access("load16_cas128", table_bytes, 1 << 30, stream.cuda_stream)
        r_l2 = swapgb.probe_random_access("load16_cas128", 48 << 20, 1 << 30, stream.cuda_stream)
        r_x4 = swapgb.probe_random_access("load16_x4", table_bytes, 1 << 29, stream.cuda_stream)
        # per read of length L: (L-k+1) key probes + 2(L-k) slot increments
        ops = n_occ + 2 * (n_occ - n_with_occ)
        count_ms = mean_ms[3] if used == swapgb.ALGO_BUCKETED else mean_ms[2]
        atomic = {"R_red_add_u32_per_s": r_red, "dram_load16_cas128_per_s": r_pat,
                  "dram_load16_per_s_4_in_flight": r_x4,
                  "l2_load16_cas128_per_s": r_l2, "table_bytes": table_bytes,
                  "ops_per_step": ops, "achieved_ops_per_s": ops / (mean_ms[4] * 1e-3),
                  # the algorithmic op count over time, against R: context only.
                  # The bucketed build does not perform these ops as random DRAM
                  # atomics, so this is no roofline fraction (see "roofline").
                  "algorithmic_ops_over_R": ops / (mean_ms[4] * 1e-3) / r_red,
                  "occurrences_per_s_counting_phase": n_occ / (count_ms * 1e-3),
                  "frac_counting_phase_vs_" + ("dram" if used == swapgb.ALGO_DIRECT else "l2")
                  + "_load16_cas128": (n_occ / (count_ms * 1e-3))
                  / (r_pat if used == swapgb.ALGO_DIRECT else r_l2)}
    batched = None
    if rank == 0 and not args.no_batch and not args.reads:
        batched = batched_metrics(stream.cuda_stream)
    served = None
    if rank == 0 and not args.no_serve and not args.reads:
        served = served_metrics(stream.cuda_stream)
    if merge and atomic:
        achieved = MERGE_RANDOM_PER_NODE * survivors / (merge["ms"] * 1e-3)
        peak = atomic["dram_load16_per_s_4_in_flight"]
        merge["roofline"] = {"bound": "random access", "achieved": achieved, "peak": peak,
                             "unit": "accesses/s", "frac": achieved / peak,
                             "peak_source": "random 16-byte loads, four in flight per thread, over a "
                                            "16 GiB table: probe of this run"}
    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        cpu = cpu_baseline(text, n_bases)
        if merge:
            merge["cpu_baseline"] = merge_cpu_baseline(g, K)

    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": "bases/s", "n_gpus": world,
            "steps": args.steps, "warmup": max(args.warmup, 3), "ms_per_step": ms_per_step,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "u64",
            "data": "synthetic (seeded generator, no dataset)", "config": config_dict(),
            "arm": {"algorithm": args.algo, "read_order": args.order,
                    "algorithm_used": {1: "direct", 2: "partitioned", 3: "bucketed"}[used],
                    "inputs": "packed 2-bit reads resident in HBM"},
            "e2e": {"value": aggregate_value(n_bases, world, e2e_s * 1e3), "unit": "bases/s",
                    "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h, "wall_ms_steps": e2e_steps,
                    # context for steps slowed outside the build (value is the mean)
                    "median_wall_ms": statistics.median(e2e_steps),
                    "value_at_median": aggregate_value(n_bases, world, statistics.median(e2e_steps)),
                    "build_event_ms_steps": e2e_build_ms_steps,
                    "path": "swg_graph_build_fasta_to_host: the pinned FASTA text framed and packed "
                            "on the device (texts of 96 MiB and more stream up in pieces), built, and "
                            "the filtered graph written into pinned host arrays as buckets are counted",
                    "two_calls": {"value": aggregate_value(n_bases, world, e2e2_s * 1e3),
                                  "wall_ms_steps": e2e2_steps,
                                  "path": "swg_graph_build_fasta + swg_graph_copy_out", "one_step": e2e_phases}},
            "e2e_packed": {"value": aggregate_value(n_bases, world, e2e_p_s * 1e3),
                           "unit": "bases/s", "h2d_bytes_per_step": h2d_p,
                           "d2h_bytes_per_step": d2h, "wall_ms_steps": e2e_p_steps,
                           "path": "swg_graph_build on pinned host packed reads + swg_graph_copy_out"},
            "dropin": dropin,
            "gpu_launches": launches,
            "build": dict(info, phase_ms_mean=mean_ms),
            "roofline": roofline,
            "random_access": atomic,
            "merge": merge,
            "batched": batched,
            "served": served,
            "cpu_baseline": cpu,
            "clocks": clocks.summary(),
            "kmers_per_s": world * n_occ / (ms_per_step * 1e-3),
            "occurrences": n_occ, "distinct": distinct, "survivors": survivors,
            "wall_s_timed_region": t_wall,
        }
        print(json.dumps(line))
    if world > 1:
        dist.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())
