"""Benchmark: tall-skinny QR through the lila C ABI on one GB300.

Workload (default): BASELINE config 2, the tall-skinny Cholesky QR +
Householder reconstruction leaf lila_dgeqrf_w03_mt_hr on A = U diag(sigma) V^T,
m = 4,194,304, n = 64, mt = 32, kappa = 1e2 (U = Q factor of a seeded Gaussian,
V Haar-random, sigma log-spaced 1 -> 1/kappa; synthetic, seeds 201/202).
One step = one factorization (V, R into A, T tiles, explicit Q) of a fresh,
already-resident copy of A; every copy is 2.1 GB, far larger than the 129 MB
L2, so no L2 flush is needed between steps.

metric value: GFLOP/s credited with the Householder count 4mn^2 - 4/3 n^3
(lila-c/main_w03.c:200), plus matrices/s.  e2e: the same call with the input
copied from pinned host memory and V/R/Q copied back inside the timed region.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
"""
import argparse
import json
import os
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
for _p in (ROOT, os.path.join(ROOT, "oracle")):
    if _p not in sys.path:
        sys.path.insert(0, _p)

METRIC = "QR GFLOP/s & mats/s at FP64-grade accuracy: mixed vs plain FP64, 1 GB300"


def credited_flops(m, n):
    return 4.0 * m * n * n - 4.0 / 3.0 * n ** 3


def load_peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return json.load(f), "measured"
    except OSError:
        return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0, "bf16_tflops_sustained": 1700.0}, "fallback"


# ---------------------------------------------------------------------------
# inputs
# ---------------------------------------------------------------------------
def make_tall_input_torch(m, n, kappa, seed_u=201, seed_v=202, device="cuda"):
    """A = U diag(sigma) V^T on the device (column-major view)."""
    import torch

    g = torch.Generator(device=device)
    g.manual_seed(seed_u)
    G = torch.randn((n, m), generator=g, dtype=torch.float64, device=device).t()  # column-major m x n
    U, _ = torch.linalg.qr(G)
    gv = torch.Generator(device=device)
    gv.manual_seed(seed_v)
    Gv = torch.randn((n, n), generator=gv, dtype=torch.float64, device=device)
    V, Rv = torch.linalg.qr(Gv)
    V = V * torch.sign(torch.diagonal(Rv)).unsqueeze(0)
    sig = torch.tensor([kappa ** (-j / (n - 1)) for j in range(n)], dtype=torch.float64, device=device)
    A = (U * sig.unsqueeze(0)) @ V.t()
    out = torch.empty((n, m), dtype=torch.float64, device=device).t()
    out.copy_(A)
    del G, U, A
    return out


def make_tall_input_numpy(m, n, kappa, seed_u=201, seed_v=202):
    import numpy as np

    rng = np.random.default_rng(seed_u)
    U, _ = np.linalg.qr(rng.standard_normal((m, n)))
    rv = np.random.default_rng(seed_v)
    V, Rv = np.linalg.qr(rv.standard_normal((n, n)))
    V = V * np.sign(np.diag(Rv))[None, :]
    sig = np.array([kappa ** (-j / (n - 1)) for j in range(n)])
    return np.asfortranarray((U * sig[None, :]) @ V.T)


# ---------------------------------------------------------------------------
# clocks
# ---------------------------------------------------------------------------
class ClockSampler:
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index=0):
        self.proc = None
        self.lines = []
        self.gpu = gpu_index

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.gpu), "--query-gpu=" + self.FIELDS, "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except OSError:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.proc is None:
            return None
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax.append(float(parts[2]))
            except ValueError:
                continue
            for nm, v in zip(names, parts[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        if not sm:
            return None
        sm.sort()
        return {"sm_mhz": sm[len(sm) // 2], "sm_max_mhz": max(smax), "reasons": sorted(reasons),
                "samples": len(sm)}


# ---------------------------------------------------------------------------
# CPU baseline (oracle restatement on OpenBLAS, or the self-contained oracle)
# ---------------------------------------------------------------------------
def cpu_baseline(m_sample, n, mt, kappa, reps=3):
    import numpy as np

    import oracle as O

    lib = O.load("oracle_ob")
    kind_note = "oracle C restatement of lila_dgeqrf_w03_mt_hr on scipy's OpenBLAS"
    if lib is None:
        lib = O.load("oracle")
        kind_note = "oracle C restatement of lila_dgeqrf_w03_mt_hr (own BLAS loops, OpenMP)"
    A0 = make_tall_input_numpy(m_sample, n, kappa)
    times = []
    for r in range(reps + 1):
        A = A0.copy(order="F")
        T = np.asfortranarray(np.zeros((mt, n)))
        Q = np.asfortranarray(np.zeros((m_sample, n)))
        work = np.zeros(lib.query_dgeqrf_w03_mt_hr(m_sample, n, 0, mt) + 16)
        t0 = time.perf_counter()
        lib.dgeqrf_w03_mt_hr(m_sample, n, 0, mt, A, m_sample, T, mt, Q, m_sample, work, work.size)
        t1 = time.perf_counter()
        if r > 0:
            times.append(t1 - t0)
    times.sort()
    t = times[len(times) // 2]
    cores = os.cpu_count()
    return {
        "value": credited_flops(m_sample, n) / t / 1e9,
        "unit": "GFLOP/s",
        "cores": cores,
        "kind": "port",
        "sample": "%s, m=%d (of 4,194,304) x n=%d, mt=%d, kappa=%g; median of %d after 1 warm-up; "
                  "OPENBLAS/OMP threads=%s" % (kind_note, m_sample, n, mt, kappa, reps,
                                               os.environ.get("OPENBLAS_NUM_THREADS", str(cores))),
        "seconds_per_matrix": t,
        "mats_per_s_scaled_to_full_m": 1.0 / (t * (4194304 / m_sample)),
    }


# ---------------------------------------------------------------------------
# GPU arm
# ---------------------------------------------------------------------------
def run_ours(args, rank, world):
    import torch

    import lila_gb300 as L

    torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
    L.lib()
    m, n, mt, kappa = args.m, args.n, args.mt, args.kappa
    base = make_tall_input_torch(m, n, kappa)
    nbuf = args.warmup + args.steps
    bufs = []
    for _ in range(nbuf):
        b = torch.empty((n, m), dtype=torch.float64, device="cuda").t()
        b.copy_(base)
        bufs.append(b)
    T = L.colmajor(mt, n, fill=0.0)
    Q = L.colmajor(m, n, fill=0.0)
    lw = L.query_dgeqrf_w03_mt_hr(m, n, 0, mt, None, m, None, mt, None, m, None, -1)
    W = torch.empty(lw, dtype=torch.float64, device="cuda")
    stream = torch.cuda.current_stream()

    def step(A):
        rc = L.dgeqrf_w03_mt_hr(m, n, 0, mt, A, m, T, mt, Q, m, W, lw)
        assert rc == 0, rc

    for s in range(args.warmup):
        step(bufs[s])
    torch.cuda.synchronize()
    if world > 1:
        import torch.distributed as dist

        dist.barrier()
    clocks = ClockSampler(int(os.environ.get("LOCAL_RANK", "0")))
    clocks.start()
    L.trace(True)
    l0 = L.launch_count()
    torch.cuda.synchronize()
    ev0 = torch.cuda.Event(enable_timing=True)
    ev1 = torch.cuda.Event(enable_timing=True)
    ev0.record(stream)
    for s in range(args.steps):
        step(bufs[args.warmup + s])
    ev1.record(stream)
    torch.cuda.synchronize()
    launches = L.launch_count() - l0
    trace = L.trace_summary()
    L.trace(False)
    clk = clocks.stop()
    ms = ev0.elapsed_time(ev1) / args.steps
    if world > 1:
        import torch.distributed as dist

        t = torch.tensor([ms], dtype=torch.float64, device="cuda")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        ms = float(t.item())
    # accuracy of the last factorization (FP64 torch products, reporting only)
    Af = bufs[args.warmup + args.steps - 1]
    R = torch.triu(Af[:n, :n])
    res = float(torch.linalg.norm(Q @ R - base) / torch.linalg.norm(base))
    orth = float(torch.linalg.norm(torch.eye(n, dtype=torch.float64, device="cuda") - Q.t() @ Q))
    status = L.gpu_status()
    del bufs

    # e2e: host buffers, copies inside the timed region
    e2e_steps = max(1, min(args.steps, 3))
    hA = torch.empty((n, m), dtype=torch.float64, pin_memory=True).t()
    hA.copy_(base.cpu())
    hA_out = torch.empty((n, m), dtype=torch.float64, pin_memory=True).t()
    hQ_out = torch.empty((n, m), dtype=torch.float64, pin_memory=True).t()
    dA = torch.empty((n, m), dtype=torch.float64, device="cuda").t()
    torch.cuda.synchronize()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(e2e_steps):
        dA.copy_(hA, non_blocking=True)
        step(dA)
        hA_out.copy_(dA, non_blocking=True)
        hQ_out.copy_(Q, non_blocking=True)
    e1.record(stream)
    torch.cuda.synchronize()
    e2e_ms = e0.elapsed_time(e1) / e2e_steps
    if world > 1:
        import torch.distributed as dist

        t = torch.tensor([e2e_ms], dtype=torch.float64, device="cuda")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        e2e_ms = float(t.item())

    flops = credited_flops(m, n)
    gflops = world * flops / (ms * 1e-3) / 1e9
    peaks, peak_src = load_peaks()
    # dominant kernel of the timed region
    dom = max(trace.items(), key=lambda kv: kv[1][1]) if trace else ("none", (1, 1.0))
    dname, (dcnt, dms) = dom
    total_traced = sum(v[1] for v in trace.values()) or 1.0
    # algorithmic bytes per launch for the kernels of this leaf (m x n tall panel, tile width mt)
    alg = {
        "cholqr_gram": 8.0 * m * n,            # read the m x n panel once
        "cholqr_trsm": 16.0 * m * n,           # read + write Q
        "hr_trsm_v": 16.0 * m * mt,            # read + write one tile of V
        "hr_couple": 24.0 * m * mt,            # read V(earlier), read + write V(tile)
        "copy2d": 16.0 * m * n * (mt / n) if dname == "copy2d" else 0.0,
        "flip_cols": 16.0 * m * mt,
    }
    bytes_per_launch = alg.get(dname, 0.0)
    achieved = bytes_per_launch / (dms / dcnt * 1e-3) / 1e9 if bytes_per_launch else None
    result = {
        "metric": METRIC,
        "value": gflops,
        "unit": "GFLOP/s",
        "mats_per_s": world * 1e3 / ms,
        "n_gpus": world,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": ms,
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f64",
        "data": "synthetic: A = U diag(sigma) V^T, U = Q of seeded N(0,1) m x n (seed 201), V Haar "
                "(seed 202), sigma log-spaced 1 -> 1/kappa",
        "config": {"workload": "tall-skinny CholQR + Householder reconstruction "
                               "(lila_dgeqrf_w03_mt_hr, plain FP64)",
                   "m": m, "n": n, "mt": mt, "kappa": kappa, "variant": "plain-fp64",
                   "l2": "inputs larger than L2 (fresh 2.1 GB copy of A per step, no flush needed)",
                   "parallelism": "replicas" if world > 1 else "single-gpu"},
        "accuracy": {"res": res, "orth": orth, "tol": 50 * n * 2.0 ** -53, "status": status},
        "roofline": {
            "bound": "hbm",
            "kernel": dname,
            "achieved": achieved,
            "peak": peaks.get("hbm_gbs"),
            "unit": "GB/s",
            "frac": (achieved / peaks["hbm_gbs"]) if achieved else None,
            "traffic": None,
            "peak_source": peak_src,
            "kernel_share_of_traced_time": dms / total_traced,
            "kernel_launches": dcnt,
            "kernel_ms_per_launch": dms / dcnt,
        },
        "kernel_times_ms": {k: v[1] / args.steps for k, v in sorted(trace.items(), key=lambda kv: -kv[1][1])},
        "e2e": {"value": world * flops / (e2e_ms * 1e-3) / 1e9, "unit": "GFLOP/s",
                "ms_per_step": e2e_ms, "h2d_bytes_per_step": 8 * m * n,
                "d2h_bytes_per_step": 16 * m * n},
        "gpu_launches": int(launches),
        "clocks": clk,
    }
    return result


def run_reference(args, rank, world):
    """CPU reference arm: the oracle restatement of the reference's mt_hr leaf on the host cores."""
    m_sample = args.cpu_m
    t_steps = []
    res = None
    for s in range(args.warmup + args.steps):
        r = cpu_baseline(m_sample, args.n, args.mt, args.kappa, reps=1)
        if s >= args.warmup:
            t_steps.append(r["seconds_per_matrix"])
        res = r
    t = sum(t_steps) / len(t_steps)
    flops = credited_flops(m_sample, args.n)
    value = flops / t / 1e9
    cb = dict(res)
    cb["value"] = value
    return {
        "metric": METRIC,
        "impl": "reference",
        "value": value,
        "unit": "GFLOP/s",
        "n_gpus": world,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": t * 1e3,
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f64",
        "data": "synthetic: A = U diag(sigma) V^T as in the GPU arm, bounded row sample",
        "config": {"workload": "tall-skinny CholQR + Householder reconstruction "
                               "(lila_dgeqrf_w03_mt_hr, plain FP64)",
                   "m": args.m, "n": args.n, "mt": args.mt, "kappa": args.kappa, "variant": "plain-fp64",
                   "cpu_sample_m": m_sample},
        "cpu_baseline": cb,
        "e2e": {"value": value, "unit": "GFLOP/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--m", type=int, default=4194304)
    ap.add_argument("--n", type=int, default=64)
    ap.add_argument("--mt", type=int, default=32)
    ap.add_argument("--kappa", type=float, default=1e2)
    ap.add_argument("--cpu-m", type=int, default=1048576)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    args = ap.parse_args()

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    if args.impl == "reference":
        if rank != 0:
            return 0
        print(json.dumps(run_reference(args, rank, world)))
        return 0
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl")
    out = run_ours(args, rank, world)
    if rank == 0:
        if world == 1 and not args.no_cpu_baseline:
            out["cpu_baseline"] = cpu_baseline(args.cpu_m, args.n, args.mt, args.kappa)
        print(json.dumps(out))
    if world > 1:
        import torch.distributed as dist

        dist.barrier()
        dist.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())
