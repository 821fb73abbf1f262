#!/usr/bin/env python
"""Benchmark: 3PC VGG16 secure inference (batch 128, uint64 shares, 26 fractional bits).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

Workload (one "step" = one secure forward of a batch): VGG16 of Piranha's
files/models/vgg16-cifar10.json with its five averagepool layers replaced by
2x2/2 maxpool, batch 128 of synthetic 32x32x3 images uniform in [0,1],
fixed-point encoded with 26 fractional bits and shared among the three
simulated parties with seeded random masks; weights are seeded
Kaiming-uniform loaded with Piranha's setPublic. All three parties run on one
GPU; the whole forward is replayed from one CUDA graph.

Timed region: K graph replays, each preceded (outside its CUDA-event pair) by
a 256 MiB write that flushes L2; device time from CUDA events on the replay
stream; wall clock bracketed by barrier + synchronize. `value` = images/s of
the device-resident replays; `e2e` = the same through pg_net_forward_host with
pinned host shares in and out (H2D + forward + D2H per step).

With --impl reference the line times Piranha's own arithmetic restated on the
CPU (the oracle; the reference's GPU build cannot be compiled here) on a
bounded sample of the same workload with all host threads.
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
sys.path.insert(0, ROOT)

BATCH = 128
FP = 26
SEED = 2024
METRIC = "3PC VGG16 secure inference img/s"
WORKLOAD = "vgg16-cifar10 (averagepool->maxpool 2x2/2), 3PC RSS, batch 128, uint64 shares, FP 26"
LIMB_FLOPS_PER_RING_MAC = 72  # 36 8-bit limb pairs x 2 flops: exact u64 MAC on fp16 tensor cores


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--form", default="auto", choices=["auto", "u64", "tc"])
    ap.add_argument("--batch", type=int, default=BATCH)
    ap.add_argument("--cpu-seconds", type=float, default=12.0, help="CPU sample budget")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-compare", action="store_true", help="skip the plain-u64-form comparison run")
    return ap.parse_args()


# ------------------------------------------------------------------ workload

def vgg16_workload(batch, seed=SEED):
    import oracle as orc
    from tests import netref

    layers = netref.vgg16_layers()
    params = netref.kaiming_uniform_params(layers, seed, FP)
    rng = np.random.default_rng(seed + 1)
    x = orc.share_random(orc.encode(rng.uniform(0, 1, batch * 3072), np.uint64, FP), np.uint64, seed=seed + 2)
    return layers, params, x


def conv_ring_macs(layers, batch):
    """Ring multiply-adds per conv layer of one forward (3 parties x concatenated K = 6 per plaintext MAC)."""
    out = {}
    for i, L in enumerate(layers):
        if L[0] == "cnn":
            H, W, Din, Dout, f, s, p = L[1:]
            P, Q = (H + 2 * p - f) // s + 1, (W + 2 * p - f) // s + 1
            out[i] = 6 * batch * P * Q * Dout * f * f * Din
    return out


# -------------------------------------------------------------------- clocks

class ClockSampler:
    def __init__(self, index=0):
        self.index = index
        self.proc = None
        self.path = None

    def start(self):
        fd, self.path = tempfile.mkstemp(suffix=".csv")
        os.close(fd)
        q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.index}", f"--query-gpu={q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except OSError:
            self.proc = None

    def stop(self):
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        rows = []
        for line in open(self.path):
            parts = [p.strip() for p in line.split(",")]
            if len(parts) >= 9:
                rows.append(parts)
        os.unlink(self.path)
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}
        sm = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({n for r in rows for n, v in zip(names, r[5:9]) if v.lower() == "active"})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(rows)}


# ------------------------------------------------------------ CPU baseline

def cpu_baseline(layers, params, x_full, batch_full, budget_s):
    """Piranha's arithmetic restated on the CPU (the oracle), timed on a sample of the batch."""
    import oracle as orc
    from tests import netref

    orc.lib()
    n_in = x_full.shape[2] // batch_full

    def run(nimg):
        x = np.ascontiguousarray(x_full[:, :, : nimg * n_in])
        t0 = time.perf_counter()
        netref.forward(layers, params, x, nimg, FP)
        return time.perf_counter() - t0

    t1 = run(1)
    imgs, secs = 1, t1
    if t1 < budget_s / 2:
        n = max(1, min(batch_full, int((budget_s - t1) / max(t1, 1e-3))))
        secs += run(n)
        imgs += n
    cores = int(os.environ.get("OMP_NUM_THREADS", os.cpu_count() or 1))
    return {"value": imgs / secs, "unit": "img/s", "cores": cores, "kind": "port",
            "sample": f"{imgs} of the {batch_full} images of the batch ({secs:.1f} s), same weights and shares"}


# ------------------------------------------------------------------ GPU arm

def run_ours(args, rank, world, local_rank):
    import torch

    import piranha_gb300 as pg

    torch.cuda.set_device(local_rank)
    dev = torch.device("cuda", local_rank)
    stream = torch.cuda.Stream(device=dev)
    batch = args.batch
    layers, params, x = vgg16_workload(batch)
    macs = conv_ring_macs(layers, batch)

    forms = {"u64": [pg.FORM_U64], "tc": [pg.FORM_LIMB_TC], "auto": [pg.FORM_LIMB_TC, pg.FORM_U64]}[args.form]
    result = None
    with torch.cuda.stream(stream):
        for form in forms:
            try:
                result = bench_form(args, pg, torch, stream, dev, form, layers, params, x, macs, batch, world)
                break
            except pg.PiranhaError as e:
                if form == forms[-1]:
                    raise
                print(f"[bench] form {form} unavailable: {e}", file=sys.stderr)
        if result and result["form"] == "limb_tc" and not args.no_compare:
            # the same workload on the plain 64-bit integer CUDA-core form, for the limb/u64 ratio
            u = bench_form(args, pg, torch, stream, dev, pg.FORM_U64, layers, params, x, macs, batch, world)
            result["compare_u64"] = {"value": u["value"], "ms_per_step": u["ms_per_step"],
                                     "conv_tflops_equiv": u["roofline"]["achieved"],
                                     "limb_over_u64": result["value"] / u["value"]}
    return result, (layers, params, x)


def bench_form(args, pg, torch, stream, dev, form, layers, params, x, macs, batch, world):
    ctx = pg.Context(dev.index, stream=stream, form=form)
    net = pg.Network(ctx, layers, batch, FP)
    for i, prm in enumerate(params):
        if prm is not None:
            net.set_params(i, pg.to_device(prm[0], dev), pg.to_device(prm[1], dev) if prm[1] is not None else None)
    net.enable_timing(True)
    net.capture()
    # inputs resident in HBM: the network's own input buffers
    ptr0 = net.input_buffers()[0]
    xin = pg.to_device(x, dev).reshape(-1)

    class _A:
        __cuda_array_interface__ = {"shape": (6 * net.in_n,), "typestr": "<i8", "data": (ptr0, False), "version": 3}

    torch.as_tensor(_A(), device=dev).copy_(xin)
    flush = torch.empty(256 << 20, dtype=torch.uint8, device=dev)
    stream.synchronize()

    for _ in range(args.warmup):
        net.forward_resident()
    stream.synchronize()

    # ------------------------------------------------------------ timed
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    layer_ms = np.zeros(len(layers))
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    sampler = ClockSampler(dev.index)
    sampler.start()
    launches0 = ctx.kernel_launches()
    comm0 = ctx.comm()
    wall0 = time.perf_counter()
    step_ms = []
    for k in range(args.steps):
        flush.fill_(k & 0xFF)  # L2 flush, outside the event pair
        ev[k][0].record(stream)
        net.forward_resident()
        ev[k][1].record(stream)
        stream.synchronize()
        step_ms.append(ev[k][0].elapsed_time(ev[k][1]))
        layer_ms += np.array(net.layer_times_ms())
    torch.cuda.synchronize()
    wall = time.perf_counter() - wall0
    if world > 1:
        torch.distributed.barrier()
    clocks = sampler.stop()
    launches = ctx.kernel_launches() - launches0
    comm1 = ctx.comm()

    dev_s = sum(step_ms) / 1e3
    if world > 1:
        t = torch.tensor([dev_s, wall], device=dev, dtype=torch.float64)
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        dev_s, wall = float(t[0]), float(t[1])
    value = world * batch * args.steps / dev_s

    # dominant kernel: the fused share-GEMM of the conv layers
    conv_idx = sorted(macs)
    conv_ms = float(sum(layer_ms[i] for i in conv_idx)) / args.steps
    conv_macs = sum(macs.values())
    achieved = conv_macs * LIMB_FLOPS_PER_RING_MAC / (conv_ms / 1e3) / 1e12
    peaks = {}
    try:
        peaks = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except OSError:
        pass
    peak = peaks.get("bf16_tflops", 1900.0)
    peak_note = "of measured" if "bf16_tflops" in peaks else "of fallback"

    # -------------------------------------------------------------- e2e
    in_host = torch.empty(6 * net.in_n, dtype=torch.int64, pin_memory=True)
    in_host.copy_(xin.cpu())
    out_host = torch.empty(6 * net.out_n, dtype=torch.int64, pin_memory=True)
    for _ in range(max(1, args.warmup)):
        net.forward_host(in_host.data_ptr(), out_host.data_ptr())
    stream.synchronize()
    e2e_ms = []
    for k in range(args.steps):
        flush.fill_(k & 0xFF)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        net.forward_host(in_host.data_ptr(), out_host.data_ptr())
        e1.record(stream)
        stream.synchronize()
        e2e_ms.append(e0.elapsed_time(e1))
    e2e_s = sum(e2e_ms) / 1e3
    if world > 1:
        t = torch.tensor([e2e_s], device=dev, dtype=torch.float64)
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        e2e_s = float(t[0])

    per_fwd_tx = (comm1["tx"][0] - comm0["tx"][0]) // args.steps
    per_fwd_rounds = (comm1["rounds"] - comm0["rounds"]) // args.steps
    out = {
        "form": "limb_tc" if form == pg.FORM_LIMB_TC else "u64",
        "value": value,
        "ms_per_step": 1e3 * dev_s / args.steps,
        "wall_s": wall,
        "e2e": {"value": world * batch * args.steps / e2e_s, "unit": "img/s",
                "h2d_bytes_per_step": 6 * net.in_n * 8, "d2h_bytes_per_step": 6 * net.out_n * 8},
        "gpu_launches": int(launches),
        "clocks": clocks,
        "roofline": {"bound": "tensor", "achieved": achieved, "peak": peak, "unit": "TFLOP/s",
                     "frac": achieved / peak, "traffic": None,
                     "kernel": "share-GEMM implicit conv (all 13 VGG16 convs)",
                     "work": f"{LIMB_FLOPS_PER_RING_MAC} limb-tensor flops per ring MAC, {conv_macs:.4g} ring MACs/forward",
                     "peak_source": f"bf16_tflops {peak_note}"},
        "comm_per_party_per_forward": {"tx_bytes": int(per_fwd_tx), "rounds": int(per_fwd_rounds)},
        "layer_ms": [round(float(v) / args.steps, 4) for v in layer_ms],
    }
    net.close()
    ctx.close()
    return out


def main():
    args = parse()
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local_rank = int(os.environ.get("LOCAL_RANK", "0"))

    if args.impl == "reference":
        if rank != 0:
            return
        layers, params, x = vgg16_workload(args.batch)
        cb = cpu_baseline(layers, params, x, args.batch, args.cpu_seconds)
        line = {"metric": METRIC, "value": cb["value"], "unit": "img/s", "impl": "reference", "n_gpus": args.gpus,
                "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * args.batch / cb["value"],
                "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "u64",
                "data": "synthetic", "config": {"workload": WORKLOAD, "global_batch": args.batch,
                                                "parallelism": "replicas"},
                "cpu_baseline": cb, "e2e": {"value": cb["value"], "unit": "img/s", "h2d_bytes_per_step": 0,
                                            "d2h_bytes_per_step": 0},
                "note": "Piranha's GPU build needs its un-vendored CUTLASS fork; this arm times the reference's "
                        "arithmetic restated on the host CPU"}
        print(json.dumps(line))
        return

    if world > 1:
        import torch

        torch.distributed.init_process_group("nccl")
    res, wl = run_ours(args, rank, world, local_rank)
    if rank != 0:
        return
    cb = None
    if world == 1 and not args.no_cpu_baseline:
        cb = cpu_baseline(*wl, args.batch, args.cpu_seconds)
    line = {
        "metric": METRIC, "value": res["value"], "unit": "img/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": res["ms_per_step"], "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "u64", "data": "synthetic",
        "config": {"workload": WORKLOAD, "global_batch": args.batch * world, "parallelism": "replicas",
                   "form": res["form"], "l2": "256 MiB write between timed steps",
                   "graph": "one CUDA graph per forward"},
        "e2e": res["e2e"], "gpu_launches": res["gpu_launches"], "clocks": res["clocks"],
        "roofline": res["roofline"], "cpu_baseline": cb,
        "comm_per_party_per_forward": res["comm_per_party_per_forward"],
        "layer_ms": res["layer_ms"],
    }
    if "compare_u64" in res:
        line["compare_u64_form"] = res["compare_u64"]
    print(json.dumps(line))


if __name__ == "__main__":
    main()
