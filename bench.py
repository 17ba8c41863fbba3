#!/usr/bin/env python
"""Benchmark of the NDTensors block-sparse contraction path on GB300.

Workload (one "step"): one QN block-sparse two-site H_eff matvec at chi = 4096,
d = 2, w = 5, 17 U(1) charge sectors: the four pairwise block-sparse
contractions L*psi, *W1, *W2, *R, each one grouped-GEMM launch, with the block
plans built once (as in a sweep).  Synthetic seeded inputs.

Headline metric: block-sparse contract GFLOP/s (algorithmic 2*M*N*K summed over
block pairs) with the Ozaki split-precision GEMM, whose relative Frobenius error
against the FP64 path is reported beside it (bar: 1e-10); the plain FP64 path
is timed in the same run.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference] [--chi 4096]

--impl reference times the reference algorithm's CPU restatement (the oracle:
per-block-pair numpy/OpenBLAS dgemm in the reference's sequential plan order) on
the host cores with all threads, same workload, same metric.
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT / "itensors.jl_gb300"))

METRIC = "block-sparse contract GFLOP/s at rel err <=1e-10: Ozaki-INT8 vs plain FP64, 1 GB300"


def peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return dict(hbm_gbs=d["hbm_gbs"], bf16=d["bf16_tflops"], bf16_sus=d.get("bf16_tflops_sustained"),
                    src="measured")
    return dict(hbm_gbs=6800.0, bf16=1900.0, bf16_sus=1700.0, src="fallback")


class ClockSampler:
    """nvidia-smi clocks/throttle reasons sampled during the timed region."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.proc = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except Exception:
            self.proc = None
        return self

    def __exit__(self, *a):
        self.out = ""
        if self.proc:
            self.proc.terminate()
            try:
                self.out, _ = self.proc.communicate(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        rows = []
        for line in (self.out or "").strip().splitlines():
            f = [x.strip() for x in line.split(",")]
            if len(f) < 9:
                continue
            try:
                rows.append(dict(sm=float(f[1]), smax=float(f[2]), hw=f[5], hwt=f[6], swt=f[7], pcap=f[8]))
            except ValueError:
                continue
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        reasons = set()
        for r in rows:
            for k, name in (("hw", "hw_slowdown"), ("hwt", "hw_thermal_slowdown"), ("swt", "sw_thermal_slowdown"),
                            ("pcap", "sw_power_cap")):
                if r[k].lower() == "active":
                    reasons.add(name)
        return {"sm_mhz": float(np.median([r["sm"] for r in rows])), "sm_max_mhz": rows[0]["smax"],
                "reasons": sorted(reasons), "samples": len(rows)}


def dist_init():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    if ws > 1:
        import torch.distributed as dist
        backend = "nccl"
        dist.init_process_group(backend)
        return dist.get_rank(), ws, int(os.environ.get("LOCAL_RANK", "0")), dist
    return 0, 1, 0, None


def oracle_matvec(net, steps_labels):
    """One H_eff matvec with the oracle (reference algorithm restated on the CPU)."""
    from oracle import blocksparse as obs
    def conv(t):
        return obs.BlockSparseTensor([tuple(i) for i in t.inds], [tuple(b) for b in t.blocks], list(t.offsets),
                                     t.data)
    L, psi, W1, W2, R = (conv(net[k]) for k in ("L", "psi", "W1", "W2", "R"))
    (l1, l2, lr), (m1, m2, mr), (n1, n2, nr), (o1, o2, orr) = steps_labels
    t, _ = obs.contract(L, l1, psi, l2, lr)
    t, _ = obs.contract(t, m1, W1, m2, mr)
    t, _ = obs.contract(t, n1, W2, n2, nr)
    t, _ = obs.contract(t, o1, R, o2, orr)
    return t


def cpu_threads():
    try:
        return len(os.sched_getaffinity(0))
    except Exception:
        return os.cpu_count() or 1


def run_reference(args):
    rank, ws, _, dist = dist_init()
    if rank != 0:
        return
    from ndtensors_gb300 import workloads as wl
    net = wl.qn_heff(chi=args.chi)
    steps_labels = wl.heff_steps()
    cores = cpu_threads()
    # flops of one matvec (algorithmic, from the oracle's own plans)
    from oracle import blocksparse as obs
    flops = matvec_flops_oracle(net, steps_labels)
    for _ in range(args.warmup):
        oracle_matvec(net, steps_labels)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        oracle_matvec(net, steps_labels)
    dt = (time.perf_counter() - t0) / args.steps
    v = flops / dt / 1e9
    line = {"impl": "reference", "metric": METRIC, "value": round(v, 3), "unit": "GFLOP/s", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(dt * 1e3, 3),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": f"qn_heff_matvec_chi{args.chi}", "chi": args.chi, "d": 2, "w": 5, "charges": 17,
                       "flops_per_step": flops},
            "cpu_baseline": {"value": round(v, 3), "unit": "GFLOP/s", "cores": cores, "kind": "port",
                             "sample": f"{args.steps} full H_eff matvecs (oracle, numpy/OpenBLAS dgemm per block pair, "
                                       f"reference sequential plan order)"},
            "e2e": {"value": round(v, 3), "unit": "GFLOP/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def matvec_flops_oracle(net, steps_labels):
    from oracle import blocksparse as obs
    def conv(t):
        return obs.BlockSparseTensor([tuple(i) for i in t.inds], [tuple(b) for b in t.blocks], list(t.offsets),
                                     t.data)
    cur = conv(net["L"])
    others = [conv(net["psi"]), conv(net["W1"]), conv(net["W2"]), conv(net["R"])]
    tot = 0
    for (a, b, c), T in zip(steps_labels, others):
        indsr, blocks_r, offs_r, nnz_r, plan = obs.contract_blockoffsets(cur, a, T, b, c)
        tot += obs.flops_of_plan(cur, a, T, b, plan)
        cur = obs.BlockSparseTensor(indsr, blocks_r, offs_r, np.zeros(nnz_r))
    return tot


def run_ours(args):
    import torch
    rank, ws, local, dist = dist_init()
    torch.cuda.set_device(local)
    import ndtensors_gb300 as nd
    from ndtensors_gb300 import workloads as wl
    dev = torch.device("cuda", local)
    net = wl.qn_heff(chi=args.chi)
    steps_labels = wl.heff_steps()
    G = {k: nd.BlockSparseTensor.from_host(net[k], local) for k in ("L", "psi", "W1", "W2", "R")}
    h = nd.handle(local)
    if args.slices:
        h.call("nd_set_ozaki_slices", int(args.slices))

    # plans (built once, as in a sweep) and flops
    plans = []
    cur = G["L"]
    rhs = [G["psi"], G["W1"], G["W2"], G["R"]]
    outs = []
    flops = 0
    for (a, b, c), T in zip(steps_labels, rhs):
        p = nd.get_plan(cur, a, T, b, c)
        flops += p.flops(cur, T)
        plans.append(p)
        out = nd.BlockSparseTensor(list(p.indsR), list(p.blocksR), list(p.offsetsR),
                                   torch.empty(max(p.nnzR, 1), dtype=torch.float64, device=dev)[:p.nnzR])
        outs.append(out)
        cur = out

    def step(prec):
        x = G["L"]
        for (a, b, c), T, p, o in zip(steps_labels, rhs, plans, outs):
            nd.contract_blocksparse(x, a, T, b, c, precision=prec, plan=p, out=o)
            x = o
        return x

    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=dev)   # 256 MB > L2 (129 MB)

    def timed(prec, k):
        ts = []
        for _ in range(k):
            flush.fill_(1.0)
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            step(prec)
            e1.record()
            ts.append((e0, e1))
        torch.cuda.synchronize()
        return [a.elapsed_time(b) for a, b in ts]

    # accuracy: Ozaki vs FP64 on the same inputs
    ref64 = step("fp64").data.clone()
    oz = step(args.precision).data.clone()
    rel_err = float(torch.linalg.norm(oz - ref64) / torch.linalg.norm(ref64))

    for _ in range(args.warmup):
        step(args.precision)
    torch.cuda.synchronize()
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    launches0 = h.launches()
    h.profile(True)
    with ClockSampler(local) as cs:
        ts = timed(args.precision, args.steps)
    prof = h.profile_read()
    h.profile(False)
    launches = h.launches() - launches0
    torch.cuda.synchronize()
    ms = float(np.sum(ts)) / args.steps
    if dist:
        t = torch.tensor([ms], device=dev)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        ms = float(t.item())
    value = ws * flops / (ms * 1e-3) / 1e9

    # plain FP64 path in the same run (fewer steps: it is ~50x slower)
    k64 = max(1, min(3, args.steps))
    ms64 = float(np.mean(timed("fp64", k64)))
    v64 = flops / (ms64 * 1e-3) / 1e9

    # roofline of the dominant kernel (tensor pipe): slice-pair products actually issued
    S = int(args.slices or 5)
    npair_levels = S * (S + 1) // 2
    gemm_n, gemm_ms = prof.get("split_gemm", (0, 0.0))
    pk = peaks()
    roof = None
    if gemm_n:
        per_launch_ms = gemm_ms / gemm_n
        tensor_flops_per_launch = npair_levels * flops / len(plans)      # average over the 4 contractions
        achieved = tensor_flops_per_launch / (per_launch_ms * 1e-3) / 1e12
        roof = {"bound": "tensor", "achieved": round(achieved, 2), "peak": pk["bf16"], "unit": "TFLOP/s",
                "frac": round(achieved / pk["bf16"], 4), "traffic": None,
                "kernel": "split_gemm (tcgen05 kind::f16, TMEM accumulators)",
                "peak_source": f"{pk['src']} bf16 dense burst",
                "units": f"{npair_levels} BF16 slice-pair products x 2MNK per block pair",
                "kernel_share_of_step": round(gemm_ms / max(1e-9, float(np.sum(ts))), 3),
                "kernels": {k: {"launches": v[0], "ms": round(v[1], 3)} for k, v in prof.items()}}

    # end to end through the public API with host buffers (plans rebuilt, as a fresh contract call does)
    pinned = {k: torch.from_numpy(np.ascontiguousarray(net[k].data)).pin_memory() for k in ("L", "psi", "W1", "W2", "R")}
    h2d = sum(int(v.numel()) * 8 for v in pinned.values())
    out_host = torch.empty(outs[-1].nnz, dtype=torch.float64).pin_memory()
    d2h = int(out_host.numel()) * 8

    def e2e_step():
        D = {k: nd.BlockSparseTensor(G[k].inds, G[k].blocks, G[k].offsets,
                                     pinned[k].to(dev, non_blocking=True)) for k in pinned}
        x = D["L"]
        for (a, b, c), key in zip(steps_labels, ("psi", "W1", "W2", "R")):
            p = nd.ContractionPlan(x, a, D[key], b, c)
            x = nd.contract_blocksparse(x, a, D[key], b, c, precision=args.precision, plan=p)
        out_host.copy_(x.data, non_blocking=True)
        torch.cuda.synchronize()

    e2e_step()
    ke = max(1, min(3, args.steps))
    t0 = time.perf_counter()
    for _ in range(ke):
        e2e_step()
    e2e_ms = (time.perf_counter() - t0) * 1e3 / ke
    e2e_v = ws * flops / (e2e_ms * 1e-3) / 1e9

    line = {"metric": METRIC, "value": round(value, 2), "unit": "GFLOP/s", "n_gpus": ws, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": round(ms, 4), "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "precision": f"ozaki-{S}slices" if args.precision == "ozaki" else args.precision,
            "data": "synthetic",
            "config": {"workload": f"qn_heff_matvec_chi{args.chi}", "chi": args.chi, "d": 2, "w": 5, "charges": 17,
                       "contractions_per_step": 4, "block_pairs": [p.npairs for p in plans],
                       "flops_per_step": flops, "l2": "flushed between steps (256 MB write)",
                       "parallelism": f"replicas x{ws}"},
            "rel_err_vs_fp64": rel_err,
            "fp64": {"value": round(v64, 2), "unit": "GFLOP/s", "ms_per_step": round(ms64, 3)},
            "speedup_vs_fp64": round(value / ws / v64, 2),
            "roofline": roof,
            "e2e": {"value": round(e2e_v, 2), "unit": "GFLOP/s", "ms_per_step": round(e2e_ms, 3),
                    "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
                    "note": "pinned-host inputs, plans rebuilt per call, result copied back"},
            "gpu_launches": launches,
            "clocks": cs.summary()}

    # CPU baseline: the oracle on the same workload, one matvec (rank 0, N=1 only)
    if rank == 0 and ws == 1 and not args.no_cpu:
        t0 = time.perf_counter()
        oracle_matvec(net, steps_labels)
        dt = time.perf_counter() - t0
        line["cpu_baseline"] = {"value": round(flops / dt / 1e9, 3), "unit": "GFLOP/s", "cores": cpu_threads(),
                                "kind": "port", "sample": "1 full H_eff matvec (oracle: numpy/OpenBLAS dgemm per "
                                                          "block pair, sequential plan order)"}
    if rank == 0:
        print(json.dumps(line), flush=True)
    if dist:
        dist.barrier()
        dist.destroy_process_group()


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--chi", type=int, default=4096)
    ap.add_argument("--precision", default="ozaki", choices=["ozaki", "bf16x3", "fp64"])
    ap.add_argument("--slices", type=int, default=0)
    ap.add_argument("--no-cpu", action="store_true")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    if args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
