#!/usr/bin/env python3
"""Benchmark of the asynchronous NOMAD SGD hot path on one GB300.

Workload: the 480,189 x 17,770 rating matrix with 100,480,507 training and 1,408,395
test ratings (user degrees Zipf(0.8), item degrees Zipf(1.1), integer ratings 1-5 from a
planted rank-20 model), k = 100, lrate 0.002, drate 0.05, reg 0.05: seeded synthetic
data with the shape of the Netflix-prize matrix (the dataset itself is not used).

One step = one epoch of the async NOMAD kernel: every training rating updated once,
column tokens passed between worker warps (one block per SM with 12 worker warps for bf16
rows, 10 for fp32: 1,824 / 1,520 workers) through device ring queues; columns long enough to set the epoch time visit
whole thread blocks.  Both storage
forms run (fp32 and bf16 with stochastic rounding); the headline value is the bf16
form.  The device-resident number (`value`) sums CUDA-event time of the K timed epoch
launches; `e2e` times the whole job through the C-ABI from host buffers (init with the
H2D copy of the ratings, K epochs each with its online training loss and a test-RMSE
read-back, then the final train and test RMSE and the factor read-back).
Test RMSE is evaluated after every epoch, outside the timed launches, as the reference
excludes testing time from training time (Code/nomad/nb_main.cpp:265-266).

`--impl reference` times the CPU restatement of the reference's updater loop (the
oracle's asynchronous float mode, every host core) on the same workload: the reference
itself needs MPI, TBB, Boost and glog, none of which exist on these machines.
"""
import argparse
import concurrent.futures as cf
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time
import zlib

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "rating updates/s & time-to-test-RMSE on 1 GB300, BF16 vs plain FP32 GPU form"
UNIT = "rating updates/s"
WORKLOAD_ID = 2
HP = dict(dim=100, lrate=0.002, drate=0.05, reg=0.05)
BYTES_PER_UPDATE = {"fp32": 2 * 100 * 4 + 8, "bf16": 2 * 100 * 2 + 8}  # w_i read+write, index, value
TARGET_FILE = os.path.join(ROOT, "tests", "golden", "workload2_fp64_rmse.json")
ASYNC_TARGET_FILE = os.path.join(ROOT, "tests", "golden", "workload2_async_fp64_rmse.json")
W3_TARGET_FILE = os.path.join(ROOT, "tests", "golden", "workload3_fp64_rmse.json")
W3_ASYNC_TARGET_FILE = os.path.join(ROOT, "tests", "golden", "workload3_async_fp64_rmse.json")
HP3 = dict(dim=100, lrate=0.0005, drate=0.05, reg=0.05)  # ratings 0-100: a smaller step
TRAFFIC_FILE = os.path.join(ROOT, "profiles", "async_kernel_traffic.json")


def log(*a):
    print(*a, file=sys.stderr, flush=True)


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--cpu-seconds", type=float, default=12.0,
                    help="wall-clock sample of the CPU baseline")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--workers", type=int, default=0)
    ap.add_argument("--wpb", type=int, default=0)
    ap.add_argument("--bps", type=int, default=0)
    ap.add_argument("--forms", default="fp32,bf16",
                    help="storage forms to run (the headline is bf16; profiling runs pick one)")
    ap.add_argument("--workload", choices=["netflix", "batched", "memory"], default="netflix",
                    help="netflix: the headline 480,189 x 17,770 workload; batched: the "
                         "4,096-problem batch; memory: the 2.74e9-rating workload (--scale "
                         "shrinks it for profiling); the last two print a separate line")
    ap.add_argument("--count", type=int, default=4096, help="problems in the batched workload")
    ap.add_argument("--no-extra", action="store_true",
                    help="skip the 1,000,990 x 624,961 precision workload, the batched workload and "
                         "the 2.74e9-rating memory-scale workload (extra keys of the headline line)")
    ap.add_argument("--no-ttt", action="store_true",
                    help="skip the time-to-target runs (fresh contexts trained to the FP64 target)")
    ap.add_argument("--scale", type=float, default=1.0,
                    help="shrink rows, columns and ratings by this factor (profiling captures "
                         "of a smaller case of the same shape; not a headline number)")
    return ap.parse_args()


# ---------------------------------------------------------------------------------
class Dist:
    """torchrun plumbing: replicas only (one independent problem per GPU)."""

    def __init__(self):
        self.world = int(os.environ.get("WORLD_SIZE", "1"))
        self.rank = int(os.environ.get("RANK", "0"))
        self.local = int(os.environ.get("LOCAL_RANK", "0"))
        self.pg = None
        if self.world > 1:
            import torch.distributed as td
            td.init_process_group(backend="gloo")
            self.pg = td

    def barrier(self):
        if self.pg:
            self.pg.barrier()

    def reduce(self, value, op):
        if not self.pg:
            return value
        import torch
        t = torch.tensor([float(value)], dtype=torch.float64)
        self.pg.all_reduce(t, op={"max": self.pg.ReduceOp.MAX, "sum": self.pg.ReduceOp.SUM}[op])
        return float(t.item())

    def close(self):
        if self.pg:
            self.pg.destroy_process_group()


class Clocks:
    """nvidia-smi sampling while the timed launches run."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device):
        self.f = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
        try:
            self.p = subprocess.Popen(["nvidia-smi", f"--query-gpu={self.Q}", "--format=csv,noheader,nounits",
                                       "-lms", "200", "-i", str(device)], stdout=self.f,
                                      stderr=subprocess.DEVNULL)
        except OSError:
            self.p = None
        self.active = False
        self.marks = []

    def mark(self, on):
        self.marks.append((time.time(), on))

    def stop(self):
        if self.p:
            self.p.terminate()
            self.p.wait()
        self.f.flush()
        self.f.seek(0)
        rows = [r.split(", ") for r in self.f.read().strip().splitlines() if r.strip()]
        os.unlink(self.f.name)
        sm = [float(r[1]) for r in rows if len(r) >= 9 and r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in rows if len(r) >= 9 and r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = set()
        for r in rows:
            if len(r) >= 9:
                for nm_, v in zip(names, r[5:9]):
                    if v.strip().lower() == "active":
                        reasons.add(nm_)
        loaded = [s for s in sm if mx and s > 0.5 * max(mx)] or sm
        return {"sm_mhz": statistics.median(loaded) if loaded else None,
                "sm_max_mhz": max(mx) if mx else None, "reasons": sorted(reasons),
                "samples": len(sm)}


def hbm_peak():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return float(json.load(f)["hbm_gbs"]), "measured"
    except (OSError, KeyError, ValueError):
        return 6800.0, "fallback"


def target_curve(path=TARGET_FILE):
    try:
        with open(path) as f:
            return json.load(f)
    except OSError:
        return None


def workload_checksum(train, test):
    """CRC-32 over the generated rating arrays (the figure the committed FP64
    trajectories carry, so that a curve is only used on the data it was made on)."""
    c = 0
    for a in (train.row_counts, train.cols, train.vals, test.row_counts, test.cols, test.vals):
        c = zlib.crc32(np.ascontiguousarray(a).view(np.uint8), c)
    return c


# ---------------------------------------------------------------------------------
def run_form(ng, train, test, precision, W, K, device, args, clocks=None):
    """Fresh context; W warm-up + K timed epochs, test RMSE after every epoch."""
    kw = dict(HP, precision=precision, mode="async", device=device, init_parts=16,
              workers=args.workers, warps_per_block=args.wpb, blocks_per_sm=args.bps)
    t0 = time.perf_counter()
    nm = ng.Nomad(train, test, **kw)
    init_s = time.perf_counter() - t0
    info = nm.info()
    epochs = []
    for e in range(W + K):
        timed = e >= W
        if timed and clocks:
            clocks.mark(True)
        st = nm.epoch(1)
        if timed and clocks:
            clocks.mark(False)
        tr, te = nm.rmse()
        epochs.append({"device_ms": st["device_ms"], "host_s": st["host_seconds"],
                       "updates": st["updates"], "hops": st["hops"],
                       "failures": st["failures"], "train_rmse": tr, "test_rmse": te})
    nm.close()
    timed = epochs[W:]
    dev_s = sum(x["device_ms"] for x in timed) / 1e3
    upd = sum(x["updates"] for x in timed)
    return {"precision": precision, "init_s": init_s, "info": info, "epochs": epochs,
            "timed_device_s": dev_s, "timed_updates": upd,
            "updates_per_s": upd / dev_s if dev_s > 0 else 0.0,
            "ms_per_step": 1e3 * dev_s / max(K, 1),
            "host_updates_per_s": upd / max(sum(x["host_s"] for x in timed), 1e-12)}


def time_to_target(ng, train, test, form, curves, checksum, device, args, hp=HP, max_epochs=40):
    """Device seconds of training until the test RMSE is within 0.5% of the FP64 oracle's
    RMSE after all of its epochs (the committed trajectories of the same workload, init
    and hyper-parameters): a fresh context trains epoch by epoch, reading the test RMSE
    after each, until it reaches 1.005 x that RMSE or `max_epochs` pass.  Reported
    against each committed FP64 oracle: `replay` (nomad_double with one worker) and,
    where committed, `async` (nomad_double with P workers, the oracle's deterministic
    event simulation).  Per oracle: the signed relative gap (GPU - oracle) / oracle at
    every epoch, its largest magnitude over all epochs and after the first, and the
    epoch and seconds at which the target is reached.  A curve made on other data (its
    workload checksum differs) is not used."""
    curves = {k: c for k, c in curves.items() if c}
    if not curves:
        return None
    bad = {k: c.get("checksum") for k, c in curves.items() if c.get("checksum") != checksum}
    if bad:
        return {"skipped": f"workload checksum {checksum} differs from the committed curves' {bad}"}
    kw = dict(hp, precision=form, mode="async", device=device, init_parts=16,
              workers=args.workers, warps_per_block=args.wpb, blocks_per_sm=args.bps)
    need = max(len(c["test_rmse"]) for c in curves.values())
    t, rm, secs = 0.0, [], []
    with ng.Nomad(train, test, **kw) as nm:
        for e in range(max_epochs):
            t += nm.epoch(1)["device_ms"] / 1e3
            rm.append(nm.rmse(train=False)[1])
            secs.append(t)
            done = [rm[-1] <= c["test_rmse"][-1] * 1.005 for c in curves.values()]
            if e + 1 >= need and all(done):
                break
    out = {"gpu_test_rmse": rm}
    for k, c in curves.items():
        ref = c["test_rmse"]
        target = ref[-1] * 1.005
        hit = next((i for i, x in enumerate(rm) if x <= target), None)
        gaps = [(g - r) / r for g, r in zip(rm, ref)]
        out[k] = {"oracle": c.get("mode"), "target_rmse": target, "oracle_epochs": len(ref),
                  "epochs": None if hit is None else hit + 1, "seconds": None if hit is None else secs[hit],
                  "gap_per_epoch": gaps, "max_gap": max(abs(g) for g in gaps),
                  "max_gap_after_first": max((abs(g) for g in gaps[1:]), default=None),
                  "gap_at_oracle_epochs": gaps[len(ref) - 1] if len(gaps) >= len(ref) else None}
    return out


def e2e_run(ng, train, test, K, device, args):
    """The whole job through the C-ABI from host buffers."""
    kw = dict(HP, precision="bf16", mode="async", device=device, init_parts=16,
              workers=args.workers, warps_per_block=args.wpb, blocks_per_sm=args.bps)
    t0 = time.perf_counter()
    nm = ng.Nomad(train, test, **kw)
    t1 = time.perf_counter()
    upd = 0
    dev_ms = 0.0
    for _ in range(K):
        st = nm.epoch(1)               # the epoch's stats carry its online training loss
        upd += st["updates"]
        dev_ms += st["device_ms"]
        nm.rmse(train=False)           # the step's metric: test RMSE
    t2 = time.perf_counter()
    nm.rmse()                          # the job's result: both RMSEs and the factors
    nm.factors()
    info = nm.info()
    nm.close()
    dt = time.perf_counter() - t0
    return {"value": upd / dt, "unit": UNIT,
            "h2d_bytes_per_step": int(info["h2d_bytes"] // max(K, 1)),
            "d2h_bytes_per_step": int(info["d2h_bytes"] // max(K, 1)),
            "seconds": dt, "setup_s": t1 - t0, "steps_s": t2 - t1, "steps_device_s": dev_ms / 1e3,
            "result_s": dt - (t2 - t0)}


def cpu_baseline(train, seconds):
    """The oracle's asynchronous float mode (the reference's updater loop restated),
    every host core, one wall-clock interval of the same workload."""
    from oracle import oracle as O
    cores = os.cpu_count() or 1
    csc = O.row_major_to_csc(train.m, train.n, train.row_counts, train.cols, train.vals)
    W, H = (x.astype(np.float32) for x in O.init_factors(train.m, train.n, HP["dim"], 12345, cores))
    st = O.async_train(csc, W, H, nthreads=cores, n_epochs=0, timeout_sec=seconds,
                       lrate=HP["lrate"], drate=HP["drate"], reg=HP["reg"], seed=12345)
    return {"value": st["updates"] / st["seconds"], "unit": UNIT, "cores": cores,
            "kind": "port",
            "sample": (f"480,189x17,770 / 100.5M-rating workload, CPU restatement of the "
                       f"reference updater (float), {cores} threads, one {seconds:.0f} s "
                       f"training interval from the reference init ({st['updates']} updates)")}


def config_block(K, W):
    return {"workload": "480,189 x 17,770, 100,480,507 train / 1,408,395 test ratings "
                        "(Zipf(0.8) users, Zipf(1.1) items, planted rank 20, ratings 1-5)",
            "dim": HP["dim"], "lrate": HP["lrate"], "drate": HP["drate"], "reg": HP["reg"],
            "step": "one epoch (every training rating updated once)",
            "mode": "async NOMAD, one worker per warp",
            "l2": "inputs larger than L2 (800 MB ratings + 96-192 MB factors per epoch)",
            "parallelism": "replicas"}


def precision_workload_run(ng, device, args):
    """The 1,000,990 x 624,961 precision workload (252.8M training ratings, Zipf(0.9)
    degrees on both sides, integer ratings 0-100): both storage forms from the same
    init, test RMSE after every epoch, against the committed FP64 oracle trajectories of
    this workload (`replay`: one worker; `async`: P workers), each used only if its
    workload checksum matches.  The first epoch is a warm-up for the timing."""
    t = time.perf_counter()
    train, test = ng.synth(3)
    gen_s = time.perf_counter() - t
    checksum = workload_checksum(train, test)
    curves = {k: c for k, c in (("replay", target_curve(W3_TARGET_FILE)),
                                ("async", target_curve(W3_ASYNC_TARGET_FILE))) if c}
    used = {k: c for k, c in curves.items() if c.get("checksum") == checksum}
    epochs = max([len(c["test_rmse"]) for c in used.values()] + [4])
    out = {"workload": "1,000,990 x 624,961, 252,800,275 train / 4,003,960 test ratings (Zipf(0.9) both "
                       "sides, integer ratings 0-100 from a planted rank-30 model)",
           **HP3, "workload_checksum": checksum, "generate_s": gen_s, "epochs": epochs}
    skipped = sorted(set(curves) - set(used))
    if skipped:
        out["oracle_skipped"] = f"workload checksum {checksum} differs from the committed {skipped} curves"
    for form in ("fp32", "bf16"):
        t0 = time.perf_counter()
        with ng.Nomad(train, test, precision=form, mode="async", device=device, init_parts=16, **HP3) as nm:
            init_s = time.perf_counter() - t0
            ms, rm = [], []
            for _ in range(epochs):
                ms.append(nm.epoch(1)["device_ms"])
                rm.append(nm.rmse(train=False)[1])
        timed = ms[1:] if len(ms) > 1 else ms
        r = {"updates_per_s": train.nnz / (sum(timed) / len(timed) / 1e3), "ms_per_epoch": sum(timed) / len(timed),
             "init_s": init_s, "test_rmse": rm}
        for k, c in used.items():
            ref = c["test_rmse"]
            target = ref[-1] * 1.005
            hit = next((i for i, x in enumerate(rm) if x <= target), None)
            gaps = [(g - o) / o for g, o in zip(rm, ref)]
            r[k] = {"oracle": c.get("mode"), "gap_per_epoch": gaps, "max_gap": max(abs(g) for g in gaps),
                    "max_gap_after_first": max((abs(g) for g in gaps[1:]), default=None),
                    "target_rmse": target, "epochs_to_target": None if hit is None else hit + 1,
                    "seconds_to_target": None if hit is None else sum(ms[:hit + 1]) / 1e3}
        r["roofline_frac"] = BYTES_PER_UPDATE[form] * r["updates_per_s"] / 1e9 / hbm_peak()[0]
        out[form] = r
        log(f"[bench] 1,000,990x624,961 {form}: {r['updates_per_s']:.4g} updates/s, {r['ms_per_epoch']:.1f} ms/epoch")
    out["bf16_over_fp32"] = out["bf16"]["updates_per_s"] / out["fp32"]["updates_per_s"]
    return out


def host_mem_available_gb():
    try:
        with open("/proc/meminfo") as f:
            for line in f:
                if line.startswith("MemAvailable:"):
                    return int(line.split()[1]) / 1e6
    except OSError:
        pass
    return 0.0


def memory_workload_run(ng, device, epochs=2, need_gb=150.0, scale=1.0, forms=("bf16", "fp32")):
    """The memory-scale workload: 50,082,603 x 39,780 with 2.74e9 training and 3.0e7 test
    ratings (item degrees Zipf(1.0), user degrees geometric with mean 55, real-valued
    ratings from a planted rank-50 model), k = 100, both storage forms: ~10 GB of bf16 /
    ~20 GB of fp32 factors and 22 GB of ratings on the device, W far larger than L2.
    Set-up needs ~60 GB of host memory (the generated file layout, then the CSC build);
    the run is skipped, with the reason, when the host has less than `need_gb` free.
    `scale` < 1 shrinks rows, columns and ratings alike (profiling captures of a smaller
    case of the same shape)."""
    avail = host_mem_available_gb()
    need_gb *= scale
    out = {"workload": "50,082,603 x 39,780, 2,740,000,000 train / 30,000,000 test ratings (Zipf(1.0) items, "
                       "geometric(55) users, planted rank 50 + N(0, 0.2^2))",
           "dim": 100, "lrate": 0.002, "drate": 0.05, "reg": 0.05, "host_mem_available_gb": avail}
    if avail < need_gb:
        out["skipped"] = f"{avail:.0f} GB of host memory free, {need_gb:.0f} GB wanted for the set-up"
        return out
    t = time.perf_counter()
    if scale == 1.0:
        train, test = ng.synth(4)
    else:
        out["scale"] = scale
        train, test = ng.synth(ng.synth_spec(4, m=int(50082603 * scale), n=int(39780 * scale),
                                             nnz_train=int(2740000000 * scale), nnz_test=int(30000000 * scale)))
    out["generate_s"] = time.perf_counter() - t
    for form in forms:
        t0 = time.perf_counter()
        with ng.Nomad(train, test, precision=form, mode="async", device=device, init_parts=16,
                      dim=100, lrate=0.002, drate=0.05, reg=0.05) as nm:
            init_s = time.perf_counter() - t0
            info = nm.info()
            ms, rm = [], []
            for _ in range(epochs):
                ms.append(nm.epoch(1)["device_ms"])
                rm.append(nm.rmse(train=False)[1])
        ups = train.nnz / (sum(ms) / len(ms) / 1e3)
        out[form] = {"updates_per_s": ups, "ms_per_epoch": sum(ms) / len(ms), "init_s": init_s,
                     "test_rmse": rm, "device_bytes": info["device_bytes"], "max_column": info["max_column"],
                     "roofline_frac": BYTES_PER_UPDATE[form] * ups / 1e9 / hbm_peak()[0]}
        log(f"[bench] 50,082,603x39,780 {form}: {ups:.4g} updates/s, {out[form]['ms_per_epoch']:.0f} ms/epoch")
    del train, test
    if "bf16" in out and "fp32" in out:
        out["bf16_over_fp32"] = out["bf16"]["updates_per_s"] / out["fp32"]["updates_per_s"]
    return out


def batched_run(ng, device, K, W, count=4096, blocks_per_sm=0):
    """The batched form: `count` independent problems of uneven shape and rank (m in
    [200, 20,000], n in [100, 5,000], density 0.5-5%, k in {16, 32, 64}), one CUDA-graph
    launch per epoch; compared with looping the single-problem path over a sample."""
    t = time.perf_counter()
    with cf.ThreadPoolExecutor(max_workers=os.cpu_count() or 1) as ex:  # one generator thread each
        probs = list(ex.map(lambda i: ng.synth_batch_problem(i, threads=1), range(count)))
    nnz = sum(p[0].nnz for p in probs)
    log(f"[bench] {count} problems ({nnz} train ratings) generated in {time.perf_counter() - t:.1f} s")
    kw = dict(lrate=0.002, drate=0.1, reg=0.05, device=device, blocks_per_sm=blocks_per_sm)
    res = {"workload": f"{count} problems, {nnz} train ratings: m logU[200, 20k], n logU[100, 5k], "
                       "density logU[0.5%, 5%], k in {16, 32, 64}, planted rank k/4",
           "lrate": 0.002, "drate": 0.1, "reg": 0.05, "steps": K, "warmup": W,
           "step": "one epoch of every problem (one graph launch)"}
    for form in ("fp32", "bf16"):
        t0 = time.perf_counter()
        b = ng.Batch(probs, precision=form, **kw)
        init_s = time.perf_counter() - t0
        b.epoch(W)
        st = b.epoch(K)
        _, te = b.rmse()
        b.close()
        e2e_s = time.perf_counter() - t0
        res[form] = {"updates_per_s": st["updates"] / (st["device_ms"] / 1e3),
                     "ms_per_epoch": st["device_ms"] / K, "init_s": init_s,
                     "e2e_updates_per_s": (W + K) * nnz / e2e_s,
                     "median_test_rmse": float(sorted(te)[len(te) // 2])}
        log(f"[bench] batched {form}: {res[form]['updates_per_s']:.4g} updates/s, "
            f"{res[form]['ms_per_epoch']:.2f} ms/epoch")
    # looping the single-problem path (one context per problem, replay schedule) on a sample
    upd, secs = 0, 0.0
    for train, test, dim in probs[:64]:
        with ng.Nomad(train, test, dim=dim, mode="replay", precision="fp32", **kw) as nm:
            st = nm.epoch(2)
        upd += st["updates"]
        secs += st["device_ms"] / 1e3
    res["looping_single_problem_path"] = {"updates_per_s": upd / secs,
                                          "sample": "first 64 problems, fp32 replay, 2 epochs",
                                          "batched_bf16_over_looping": res["bf16"]["updates_per_s"] / (upd / secs)}
    return res


# ---------------------------------------------------------------------------------
def main_reference(args, dist):
    if dist.rank != 0:
        return
    from oracle import oracle as O  # the oracle and the workload generator; no GPU library
    train, _ = O.workload(WORKLOAD_ID)
    cores = os.cpu_count() or 1
    csc = O.row_major_to_csc(train["m"], train["n"], train["row_counts"], train["cols"], train["vals"])
    W, H = (x.astype(np.float32) for x in O.init_factors(train["m"], train["n"], HP["dim"], 12345, cores))
    sample_s = max(1.0, min(10.0, 150.0 / max(args.steps + args.warmup, 1)))
    for _ in range(args.warmup):
        O.async_train(csc, W, H, nthreads=cores, timeout_sec=sample_s, lrate=HP["lrate"],
                      drate=HP["drate"], reg=HP["reg"])
    upd, secs = 0, 0.0
    for _ in range(args.steps):
        st = O.async_train(csc, W, H, nthreads=cores, timeout_sec=sample_s, lrate=HP["lrate"],
                           drate=HP["drate"], reg=HP["reg"])
        upd += st["updates"]
        secs += st["seconds"]
    v = upd / secs
    sample = (f"{args.steps} training intervals of {sample_s:.1f} s each on the 480,189x17,770 "
              f"workload, {cores} threads, CPU restatement of the reference updater (float)")
    print(json.dumps({
        "impl": "reference", "metric": METRIC, "value": v, "unit": UNIT, "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": 1e3 * secs / max(args.steps, 1), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": config_block(args.steps, args.warmup),
        "cpu_baseline": {"value": v, "unit": UNIT, "cores": cores, "kind": "port",
                         "sample": sample},
        "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "note": "the reference's updater compiles only where its source tree is (against "
                "stand-ins for MPI, TBB, Boost and glog); the GPU host has no copy of it, so "
                "this is the oracle's restatement of its updater loop, inputs made by the "
                "standalone workload generator (no GPU library loaded)"}), flush=True)


def main_ours(args, dist):
    import nomad_gb300 as ng
    device = dist.local
    if not ng.device_ok(device):
        raise SystemExit(f"cuda:{device} is not an sm_103 device")
    K, W = args.steps, args.warmup
    t = time.perf_counter()
    if args.scale == 1.0:
        train, test = ng.synth(WORKLOAD_ID)
    else:
        s = args.scale
        train, test = ng.synth(ng.synth_spec(WORKLOAD_ID, m=int(480189 * s), n=int(17770 * s),
                                             nnz_train=int(100480507 * s), nnz_test=int(1408395 * s)))
    log(f"[bench] workload generated in {time.perf_counter() - t:.1f} s "
        f"(nnz {train.nnz} / {test.nnz})")
    clocks = Clocks(device)
    dist.barrier()
    res = {}
    forms = [f for f in ("fp32", "bf16") if f in args.forms.split(",")]
    for form in forms:
        res[form] = run_form(ng, train, test, form, W, K, device, args,
                             clocks if form == forms[-1] else None)
        log(f"[bench] {form}: {res[form]['updates_per_s']:.4g} updates/s, "
            f"{res[form]['ms_per_step']:.2f} ms/epoch, test RMSE "
            f"{res[form]['epochs'][-1]['test_rmse']:.5f}, init {res[form]['init_s']:.1f} s")
    clk = clocks.stop()
    dist.barrier()
    if args.scale != 1.0 or len(forms) < 2:  # a profiling run: no headline line
        log(json.dumps({f: {"updates_per_s": r["updates_per_s"], "ms_per_step": r["ms_per_step"]}
                        for f, r in res.items()}))
        return
    b = res["bf16"]
    # whole-job aggregate over ranks: updates summed, time = slowest rank
    tot_upd = dist.reduce(b["timed_updates"], "sum")
    max_s = dist.reduce(b["timed_device_s"], "max")
    value = tot_upd / max_s
    e2e = None if args.no_e2e else e2e_run(ng, train, test, K, device, args)
    if e2e and dist.world > 1:
        e2e["value"] = dist.reduce(e2e["value"], "sum")
    peak, peak_kind = hbm_peak()
    achieved = BYTES_PER_UPDATE["bf16"] * b["timed_updates"] / b["timed_device_s"] / 1e9
    traffic = None
    try:
        with open(TRAFFIC_FILE) as f:
            tr = json.load(f)
        traffic = tr["dram_bytes_per_update"]["bf16"] * b["timed_updates"] / max(K, 1)
    except (OSError, KeyError, ValueError):
        pass
    checksum = workload_checksum(train, test)
    curves = {"replay": target_curve(TARGET_FILE), "async": target_curve(ASYNC_TARGET_FILE)}
    ttt = None if args.no_ttt else {f: time_to_target(ng, train, test, f, curves, checksum, device, args)
                                    for f in forms}
    extra = {}
    if not args.no_extra and dist.world == 1:
        extra["precision_workload"] = precision_workload_run(ng, device, args)
        extra["batched"] = batched_run(ng, device, K=6, W=2)
        extra["memory_workload"] = memory_workload_run(ng, device)
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": dist.world,
        "steps": K, "warmup": W, "ms_per_step": b["ms_per_step"], "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "bf16",
        "compute_dtype": "f32 (bf16 storage, stochastic-rounding write-back)",
        "data": "synthetic (seeded, shape of the 480,189x17,770 Netflix-prize matrix)",
        "config": config_block(K, W),
        "fp32": {"value": res["fp32"]["updates_per_s"], "ms_per_step": res["fp32"]["ms_per_step"],
                 "roofline_frac": BYTES_PER_UPDATE["fp32"] * res["fp32"]["updates_per_s"] / 1e9 / peak,
                 "final_test_rmse": res["fp32"]["epochs"][-1]["test_rmse"]},
        "bf16_over_fp32": b["updates_per_s"] / res["fp32"]["updates_per_s"],
        "final_test_rmse": b["epochs"][-1]["test_rmse"],
        "time_to_target": ttt,
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": achieved / peak, "traffic": traffic,
                     "peak_source": f"of {peak_kind}",
                     "bytes_per_update": BYTES_PER_UPDATE["bf16"],
                     "kernel": "nomad_async2_kernel<bf16> (one launch per epoch)"},
        "clocks": clk,
        "e2e": e2e,
        # per timed epoch: the queue seeding kernel, the tail advance and the async kernel
        "gpu_launches": 3 * K,
        "workers": b["info"]["workers"], "segments_per_epoch": b["info"]["segments"],
        "max_column": b["info"]["max_column"],
        "host_updates_per_s": b["host_updates_per_s"],
        "workload_checksum": checksum,
        **extra,
    }
    if dist.rank == 0 and dist.world == 1 and not args.no_cpu:
        line["cpu_baseline"] = cpu_baseline(train, args.cpu_seconds)
    if dist.rank == 0:
        print(json.dumps(line), flush=True)


def main_batched(args, dist):
    """The batched form: `count` independent problems of uneven shape and rank (m in
    [200, 20,000], n in [100, 5,000], density 0.5-5%, k in {16, 32, 64}), one CUDA-graph
    launch per epoch; compared with looping the single-problem path over a sample."""
    import nomad_gb300 as ng
    K, W = args.steps, args.warmup
    res = batched_run(ng, dist.local, K, W, args.count, args.bps)
    b = res["bf16"]
    print(json.dumps({
        "metric": "aggregate rating updates/s, batched independent problems", "value": b["updates_per_s"],
        "unit": UNIT, "n_gpus": dist.world, "steps": K, "warmup": W, "ms_per_step": b["ms_per_epoch"],
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "bf16",
        "data": "synthetic (seeded batched workload)",
        "config": {k: res[k] for k in ("workload", "lrate", "drate", "reg", "step")},
        "fp32": res["fp32"], "bf16": res["bf16"],
        "looping_single_problem_path": res["looping_single_problem_path"],
        "e2e": {"value": b["e2e_updates_per_s"], "unit": UNIT}}), flush=True)


def main():
    args = parse()
    dist = Dist()
    try:
        if args.impl == "reference":
            main_reference(args, dist)
        elif args.workload == "batched":
            main_batched(args, dist)
        elif args.workload == "memory":
            import nomad_gb300 as ng
            forms = tuple(f for f in ("bf16", "fp32") if f in args.forms.split(","))
            print(json.dumps(memory_workload_run(ng, dist.local, epochs=max(args.steps, 1), scale=args.scale,
                                                 forms=forms)), flush=True)
        else:
            main_ours(args, dist)
    finally:
        dist.close()


if __name__ == "__main__":
    main()
