#!/usr/bin/env python
"""Benchmark: 3PC VGG16 secure inference (batch 128, uint64 shares, 26 fractional bits).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference] [--workload NAME]

Default workload (one "step" = one secure forward of a batch): VGG16 of
Piranha's files/models/vgg16-cifar10.json with its five averagepool layers
replaced by 2x2/2 maxpool, batch 128 of synthetic 32x32x3 images uniform in
[0,1], fixed-point encoded with 26 fractional bits and shared among the three
simulated parties with seeded random masks; weights are seeded
Kaiming-uniform loaded with Piranha's setPublic. All three parties run on one
GPU; the whole forward is replayed from one CUDA graph.

Timed region: K graph replays, each preceded (outside its CUDA-event pair) by
a 256 MiB write that flushes L2; device time from CUDA events on the replay
stream; wall clock bracketed by barrier + synchronize. `value` = images/s of
the device-resident replays; `e2e` = the same through pg_net_forward_host with
pinned host shares in and out (H2D + forward + D2H per step).

Other workloads (--workload), each printing the same JSON line for its own metric:
  secureml      3PC SecureML (784-128-128-10, ReLU after every FC) inference, batch 128, u64, FP 26
  lenet-train   3PC LeNet training step (forward + backward + SGD, log learning rate 5), batch 128
  vgg16-train   3PC VGG16 training step (the reference's vgg16-cifar10 with averagepool), batch 128
  secureml-2pc  2PC SecureML inference, batch 128, uint32 shares, FP 10
  secureml-4pc  4PC SecureML inference, batch 128, uint32 shares, FP 10
  stream        512 requests of batch 1..64, SecureML or VGG16, served in order; p50/p99 latency
  gemm          3PC share-GEMM M = N = K = 4096 with truncation by 2^26 (the matmul's dividePublic3out3
                and reshare), uniform random uint64 shares; --sweep adds M = N = K in 512..8192 and five
                non-cubic (M, N, K) in that range

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
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

from piranha_gb300 import encode as enc  # noqa: E402
from piranha_gb300 import nets  # noqa: E402

BATCH = 128
SEED = 2024
LIMB_FLOPS_PER_RING_MAC = 72  # 36 8-bit limb pairs x 2 flops: exact u64 MAC on fp16 tensor cores
# DRAM bytes read + written by the 13 limb_tma_kernel launches of one VGG16
# batch-128 forward, from one ncu capture of dram__bytes_read.sum +
# dram__bytes_write.sum over those launches (bench.py --steps 1 --warmup 3
# --form tc under ncu with the plain run's tuning cache)
VGG16_B128_LIMB_TRAFFIC = 5_513_132_544

WORKLOADS = {
    "vgg16": {"metric": "3PC VGG16 secure inference img/s", "kind": "infer3", "fp": 26, "ring": "u64",
              "desc": "vgg16-cifar10 (averagepool->maxpool 2x2/2), 3PC RSS, batch 128, uint64 shares, FP 26"},
    "secureml": {"metric": "3PC SecureML secure inference img/s", "kind": "infer3", "fp": 26, "ring": "u64",
                 "desc": "secureml 784-128-128-10 (ReLU after every FC), 3PC RSS, batch 128, uint64 shares, FP 26"},
    "lenet-train": {"metric": "3PC LeNet training step img/s", "kind": "train3", "fp": 26, "ring": "u64",
                    "log_lr": 5,
                    "desc": "lenet (maxpool variant), 3PC RSS, batch 128, uint64 shares, FP 26, "
                            "forward + revealed-softmax backward + SGD (log learning rate 5)"},
    "vgg16-train": {"metric": "3PC VGG16 training step img/s", "kind": "train3", "fp": 26, "ring": "u64",
                    "log_lr": 5,
                    "desc": "vgg16-cifar10 as the reference trains it (five 2x2/2 averagepools), 3PC RSS, batch 128, "
                            "uint64 shares, FP 26, forward + revealed-softmax backward + SGD (log learning rate 5)"},
    "secureml-2pc": {"metric": "2PC SecureML secure inference img/s", "kind": "fcnet", "parties": 2, "fp": 10,
                     "ring": "u32",
                     "desc": "secureml 784-128-128-10, 2PC (TPC), batch 128, uint32 shares, FP 10"},
    "secureml-4pc": {"metric": "4PC SecureML secure inference img/s", "kind": "fcnet", "parties": 4, "fp": 10,
                     "ring": "u32",
                     "desc": "secureml 784-128-128-10, 4PC (FPC), batch 128, uint32 shares, FP 10"},
    "gemm": {"metric": "3PC share-GEMM ring MAC/s", "kind": "gemm", "fp": 26, "ring": "u64", "M": 4096, "N": 4096,
             "K": 4096, "unit": "ring-MAC/s",
             "desc": "3PC RSS matmul M=N=K=4096 over Z_2^64 (uniform random shares), truncation by 2^26 and "
                     "reshare; 6*M*N*K ring multiply-adds per step (3 parties x the concatenated K)"},
    "conv": {"metric": "3PC share-convolution ring MAC/s", "kind": "conv", "fp": 26, "ring": "u64",
             "unit": "ring-MAC/s",
             "desc": "3PC RSS convolution (fprop) of one VGG16-shaped layer (--conv-shape H,W,Din,Dout,f,stride,pad; "
                     "default 32,32,64,64,3,1,1), uniform random uint64 shares, truncation by 2^26; "
                     "6*batch*P*Q*Dout*f*f*Din ring multiply-adds per step"},
    "stream": {"metric": "3PC batched request stream img/s", "kind": "stream", "fp": 26, "ring": "u64",
               "requests": 512, "max_batch": 64,
               "desc": "512 requests, batch uniform in 1..64, SecureML or VGG16 (even odds), 3PC RSS, uint64 "
                       "shares, FP 26; waiting requests of one model are packed (up to 128 images) into one "
                       "replay of a captured network whose batch bucket (1, 2, 4, 6, 8, 12, 16, 24, ..., 64, 80, "
                       "96, 112, 128) holds them: the smallest, or a larger one of the model that replays faster"},
}
_LAYERS = {"vgg16": nets.vgg16, "secureml": nets.secureml, "lenet-train": nets.lenet,
           "vgg16-train": lambda: nets.vgg16(maxpool=False),
           "secureml-2pc": nets.secureml, "secureml-4pc": nets.secureml, "stream": nets.vgg16}


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="vgg16", choices=sorted(WORKLOADS))
    ap.add_argument("--form", default="auto", choices=["auto", "u64", "tc"])
    ap.add_argument("--batch", type=int, default=BATCH)
    ap.add_argument("--cpu-seconds", type=float, default=12.0, help="CPU sample budget of the cpu_baseline key")
    ap.add_argument("--ref-seconds", type=float, default=120.0,
                    help="--impl reference: bound on the timed CPU steps' total time")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-compare", action="store_true", help="skip the plain-u64-form comparison run")
    ap.add_argument("--sweep", action="store_true", help="gemm: also time M = N = K in 512..8192 and five non-cubic shapes in both forms")
    ap.add_argument("--no-autotune", action="store_true", help="split-K by the heuristic instead of by timing")
    ap.add_argument("--conv-shape", default="32,32,64,64,3,1,1", help="conv: H,W,Din,Dout,f,stride,pad")
    ap.add_argument("--no-pack", action="store_true", help="stream: one request per replay")
    return ap.parse_args()


# ------------------------------------------------------------------ workload

def make_workload(name, batch, seed=SEED):
    """Layers, setPublic-loaded seeded parameters, seeded input shares (and labels for training)."""
    w = WORKLOADS[name]
    layers = _LAYERS[name]()
    fp, ring = w["fp"], w["ring"]
    rng = np.random.default_rng(seed + 1)
    vals = rng.uniform(0, 1, batch * nets.input_size(layers))
    if w["kind"] == "fcnet":
        setp = enc.tpc_set_public if w["parties"] == 2 else enc.fpc_set_public
        prng = np.random.default_rng(seed)
        params = []
        for L in layers:
            if L[0] == "fc":
                din, dout = L[1], L[2]
                wv = prng.uniform(-1, 1, din * dout) * np.sqrt(6.0 / din)
                params.append((setp(wv, ring, fp), setp(np.full(dout, 0.01), ring, fp)))
            else:
                params.append(None)
        return {"layers": layers, "params": params, "x": setp(vals, ring, fp), "labels": None}
    params = nets.kaiming_uniform(layers, seed, fp)
    x = enc.share_random(enc.encode(vals, ring, fp), ring, seed=seed + 2)
    labels = None
    if w["kind"] == "train3":
        classes = np.random.default_rng(seed + 3).integers(0, 10, batch)
        labels = enc.set_public(enc.one_hot(classes, 10), ring, fp)
    return {"layers": layers, "params": params, "x": x, "labels": labels}


def make_gemm(seed=SEED):
    """Uniform random uint64 share views of A (M x K) and B (K x N), row-major."""
    w = WORKLOADS["gemm"]
    M, N, K = w["M"], w["N"], w["K"]
    rng = np.random.default_rng(seed + 11)
    A = rng.integers(0, 2**64 - 1, size=(3, 2, M * K), dtype=np.uint64, endpoint=True)
    B = rng.integers(0, 2**64 - 1, size=(3, 2, K * N), dtype=np.uint64, endpoint=True)
    return {"A": A, "B": B, "M": M, "N": N, "K": K}


def conv_geometry(args):
    H, W, Din, Dout, f, st, pd = (int(x) for x in args.conv_shape.split(","))
    P, Q = (H + 2 * pd - f) // st + 1, (W + 2 * pd - f) // st + 1
    return {"H": H, "W": W, "Din": Din, "Dout": Dout, "f": f, "stride": st, "pad": pd, "P": P, "Q": Q,
            "batch": args.batch}


def make_conv(args, seed=SEED):
    """Uniform random uint64 share views of the layer's input (NHWC) and filters (KRSC)."""
    g = conv_geometry(args)
    rng = np.random.default_rng(seed + 13)
    X = rng.integers(0, 2**64 - 1, size=(3, 2, g["batch"] * g["H"] * g["W"] * g["Din"]), dtype=np.uint64,
                     endpoint=True)
    F = rng.integers(0, 2**64 - 1, size=(3, 2, g["Dout"] * g["f"] * g["f"] * g["Din"]), dtype=np.uint64,
                     endpoint=True)
    return {**g, "X": X, "F": F}


def conv_macs(g):
    return 6 * g["batch"] * g["P"] * g["Q"] * g["Dout"] * g["f"] * g["f"] * g["Din"]


def work_per_step(name, batch):
    """Units of the workload's metric in one step: images, or ring MACs of the share-GEMM."""
    w = WORKLOADS[name]
    if w["kind"] == "gemm":
        return 6 * w["M"] * w["N"] * w["K"]
    return batch


def make_stream(seed=SEED):
    """Seeded requests: (model, batch, input shares); one parameter set per model."""
    w = WORKLOADS["stream"]
    rng = np.random.default_rng(seed + 7)
    models = {"secureml": nets.secureml(), "vgg16": nets.vgg16()}
    params = {m: nets.kaiming_uniform(L, seed, w["fp"]) for m, L in models.items()}
    reqs = []
    for r in range(w["requests"]):
        m = "secureml" if rng.integers(0, 2) == 0 else "vgg16"
        b = int(rng.integers(1, w["max_batch"] + 1))
        vals = rng.uniform(0, 1, b * nets.input_size(models[m]))
        reqs.append((m, b, enc.share_random(enc.encode(vals, "u64", w["fp"]), "u64", seed=seed + 100 + r)))
    return models, params, reqs


def ring_macs(layers, batch):
    """Ring multiply-adds per share-GEMM layer of one forward (3 parties x concatenated K = 6 per plaintext MAC)."""
    out = {}
    for i, L in enumerate(layers):
        if L[0] == "cnn":
            H, W, Din, Dout, f, s, p = L[1:]
            P, Q = (H + 2 * p - f) // s + 1, (W + 2 * p - f) // s + 1
            out[i] = 6 * batch * P * Q * Dout * f * f * Din
        elif L[0] == "fc":
            out[i] = 6 * batch * L[1] * L[2]
    return out


def executed_ring_macs(layers, batch, posmajor):
    """Ring multiply-adds the limb kernels execute per share-GEMM layer: the
    dense count, except for the convolutions the network runs with
    position-major tiles (posmajor[i], from pg_net_layer_plan), which run only
    the taps inside the input: (sum over output rows of the valid filter
    rows) x (the same over columns) taps instead of P * Q * f * f."""
    out = ring_macs(layers, batch)
    for i, L in enumerate(layers):
        if L[0] != "cnn":
            continue
        H, W, Din, Dout, f, s, p = L[1:]
        if posmajor[i]:
            rows = sum(min(f - 1, H - 1 + p - h) - max(0, p - h) + 1 for h in range(H))
            cols = sum(min(f - 1, W - 1 + p - w) - max(0, p - w) + 1 for w in range(W))
            out[i] = 6 * batch * rows * cols * Dout * Din
    return out


def load_peaks():
    try:
        return json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except OSError:
        return {}


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
                                          "--format=csv,noheader,nounits", "-lms", "50"],
                                         stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except OSError:
            self.proc = None
            return
        # the timed region starts once the sampler is up (its first line is
        # written), so a short region is covered from its start; bounded at 3 s
        t0 = time.time()
        while time.time() - t0 < 3 and self.proc.poll() is None and os.path.getsize(self.path) == 0:
            time.sleep(0.01)

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

def cpu_baseline_stream(wl, budget_s):
    """The oracle's time per image of each model (SecureML on its first
    request, VGG16 on one image of its first), applied to the stream's mix."""
    import oracle as orc
    from oracle import netref

    orc.lib()
    models, params, reqs = wl
    fp = WORKLOADS["stream"]["fp"]
    per_img = {}
    for m in models:
        _, b, x = next(r for r in reqs if r[0] == m)
        nimg = b if m == "secureml" else 1
        n_in = nets.input_size(models[m])
        t0 = time.perf_counter()
        netref.forward(models[m], params[m], np.ascontiguousarray(x[..., : nimg * n_in]), nimg, fp)
        per_img[m] = (time.perf_counter() - t0) / nimg
    imgs = sum(b for _, b, _ in reqs)
    est = sum(b * per_img[m] for m, b, _ in reqs)
    cores = int(os.environ.get("OMP_NUM_THREADS", os.cpu_count() or 1))
    return {"value": imgs / est, "unit": "img/s", "cores": cores, "kind": "port",
            "sample": "seconds per image measured on " +
                      ", ".join(f"{m} ({v:.3g} s/img)" for m, v in per_img.items()) +
                      f", applied to the stream's {imgs} images"}


def cpu_baseline_gemm(wl, budget_s):
    """The oracle's share matmul (OpenMP) on the first rows of A, extrapolated per ring MAC."""
    import oracle as orc

    M, N, K = wl["M"], wl["N"], wl["K"]
    fp = WORKLOADS["gemm"]["fp"]

    def run(rows):
        a = np.ascontiguousarray(wl["A"][..., : rows * K])
        t0 = time.perf_counter()
        orc.matmul(a, wl["B"], rows, N, K, 1, 1, 1, fp)
        return time.perf_counter() - t0

    cores = int(os.environ.get("OMP_NUM_THREADS", os.cpu_count() or 1))
    first = min(M, cores)  # one row per thread
    t1 = run(first)
    runs, secs = [first], t1
    if t1 < budget_s / 2:
        rows = max(1, min(M, int(first * (budget_s - t1) / max(t1, 1e-3)) // first * first))
        secs += run(rows)
        runs.append(rows)
    macs = sum(6 * r * N * K for r in runs)
    return {"value": macs / secs, "unit": "ring-MAC/s", "cores": cores, "kind": "port",
            "sample": f"runs of {' and '.join(map(str, runs))} rows of the {M} x {N} x {K} share matmul "
                      f"({secs:.1f} s), same shares"}


def cpu_baseline(name, wl, batch_full, budget_s):
    """Piranha's arithmetic restated on the CPU (the oracle), timed on a sample of the batch."""
    import oracle as orc
    from oracle import netref

    orc.lib()
    if name == "stream":
        return cpu_baseline_stream(wl, budget_s)
    if WORKLOADS[name]["kind"] == "gemm":
        return cpu_baseline_gemm(wl, budget_s)
    if WORKLOADS[name]["kind"] == "conv":
        g = wl
        n_img_in = g["H"] * g["W"] * g["Din"]
        t0 = time.perf_counter()
        orc.convolution(np.ascontiguousarray(g["X"][..., :n_img_in]), g["F"], orc.FPROP, 1, g["H"], g["W"], g["f"],
                        g["Din"], g["Dout"], g["stride"], g["pad"], WORKLOADS[name]["fp"])
        secs = time.perf_counter() - t0
        cores = int(os.environ.get("OMP_NUM_THREADS", os.cpu_count() or 1))
        return {"value": conv_macs(g) / g["batch"] / secs, "unit": "ring-MAC/s", "cores": cores, "kind": "port",
                "sample": f"one image of the {g['batch']}-image batch ({secs:.2f} s), same shares"}
    w = WORKLOADS[name]
    layers, params, x_full = wl["layers"], wl["params"], wl["x"]
    n_in = nets.input_size(layers)
    fp = w["fp"]

    def run(nimg):
        x = np.ascontiguousarray(x_full[..., : nimg * n_in])
        t0 = time.perf_counter()
        if w["kind"] == "infer3":
            netref.forward(layers, params, x, nimg, fp)
        elif w["kind"] == "train3":
            lab = np.ascontiguousarray(wl["labels"][..., : nimg * 10])
            netref.train_step(layers, params, x, lab, nimg, fp, w["log_lr"])
        else:
            mm = orc.tpc_matmul if w["parties"] == 2 else orc.fpc_matmul
            relu = orc.tpc_relu if w["parties"] == 2 else orc.fpc_relu
            cur = x
            for L, prm in zip(layers, params):
                if L[0] == "fc":
                    cur = mm(cur, prm[0], nimg, L[2], L[1], 1, 1, 1, fp)
                    cur = (cur.reshape(cur.shape[:-1] + (nimg, L[2])) + prm[1][..., None, :]).reshape(
                        cur.shape).astype(cur.dtype)
                else:
                    cur, _ = relu(cur)
        return time.perf_counter() - t0

    first = 2 if w["kind"] == "train3" else 1  # a training sample needs the batch division
    t1 = run(first)
    runs, secs = [first], t1
    if t1 < budget_s / 2:
        n = max(first, min(batch_full, int(first * (budget_s - t1) / max(t1, 1e-3))))
        secs += run(n)
        runs.append(n)
    imgs = sum(runs)
    cores = int(os.environ.get("OMP_NUM_THREADS", os.cpu_count() or 1))
    return {"value": imgs / secs, "unit": "img/s", "cores": cores, "kind": "port",
            "sample": f"runs of {' and '.join(map(str, runs))} images from the {batch_full}-image batch "
                      f"({secs:.1f} s), same weights and shares"}


# ------------------------------------------------------- reference arm

def reference_arm(args, name, wl):
    """--impl reference: Piranha's arithmetic restated on the CPU (the oracle,
    OpenMP over all host threads), timed step by step on the same workload.

    A step processes `per_step` units of the workload (images; share-GEMM rows
    for the gemm workload; the next request's images for the stream), taken in
    order and cycling through the batch, so that the timed steps cover the
    whole batch once when the time bound (--ref-seconds) allows it. Warm-up
    steps process the smallest unit and give the time estimate that sizes
    per_step. Every figure printed is measured, none extrapolated."""
    import oracle as orc
    from oracle import netref

    orc.lib()
    w = WORKLOADS[name]
    kind = w["kind"]
    fp = w["fp"]
    if kind == "gemm":
        M, N, K = wl["M"], wl["N"], wl["K"]
        A4 = wl["A"].reshape(3, 2, M, K)
        total, unit_work, smallest = M, 6 * N * K, min(M, os.cpu_count() or 1)

        def run(k0, n):
            rows = (k0 + np.arange(n)) % M
            a = np.ascontiguousarray(A4[:, :, rows, :].reshape(3, 2, -1))
            orc.matmul(a, wl["B"], n, N, K, 1, 1, 1, fp)
            return n
    elif kind == "conv":
        g = wl
        n_img_in = g["H"] * g["W"] * g["Din"]
        X4 = g["X"].reshape(3, 2, g["batch"], n_img_in)
        total, unit_work, smallest = g["batch"], conv_macs(g) // g["batch"], 1

        def run(k0, n):
            idx = (k0 + np.arange(n)) % g["batch"]
            x = np.ascontiguousarray(X4[:, :, idx, :].reshape(3, 2, -1))
            orc.convolution(x, g["F"], orc.FPROP, n, g["H"], g["W"], g["f"], g["Din"], g["Dout"], g["stride"],
                            g["pad"], fp)
            return n
    elif kind == "stream":
        models, params, reqs = wl
        total, unit_work, smallest = sum(b for _, b, _ in reqs), 1, 1
        state = {"req": 0}

        def run(k0, n):
            m, b, x = reqs[state["req"] % len(reqs)]
            state["req"] += 1
            nimg = min(b, n)
            n_in = nets.input_size(models[m])
            netref.forward(models[m], params[m], np.ascontiguousarray(x[..., : nimg * n_in]), nimg, fp)
            return nimg
    else:
        layers, params, x_full = wl["layers"], wl["params"], wl["x"]
        batch = args.batch
        n_in = nets.input_size(layers)
        total, unit_work = batch, 1
        smallest = 2 if kind == "train3" else 1  # a training step divides by its batch size
        xv = x_full.reshape(x_full.shape[:-1] + (batch, n_in))

        def run(k0, n):
            idx = (k0 + np.arange(n)) % batch
            x = np.ascontiguousarray(xv[..., idx, :].reshape(x_full.shape[:-1] + (-1,)))
            if kind == "infer3":
                netref.forward(layers, params, x, n, fp)
            elif kind == "train3":
                lab = np.ascontiguousarray(wl["labels"].reshape(3, 2, batch, 10)[:, :, idx, :].reshape(3, 2, -1))
                netref.train_step(layers, params, x, lab, n, fp, w["log_lr"])
            else:
                mm = orc.tpc_matmul if w["parties"] == 2 else orc.fpc_matmul
                relu = orc.tpc_relu if w["parties"] == 2 else orc.fpc_relu
                cur = x
                for L, prm in zip(layers, params):
                    if L[0] == "fc":
                        cur = mm(cur, prm[0], n, L[2], L[1], 1, 1, 1, fp)
                        cur = (cur.reshape(cur.shape[:-1] + (n, L[2])) + prm[1][..., None, :]).reshape(
                            cur.shape).astype(cur.dtype)
                    else:
                        cur, _ = relu(cur)
            return n

    est = None
    for i in range(max(1, args.warmup)):
        t0 = time.perf_counter()
        run(0, smallest)
        if i == 0:
            est = (time.perf_counter() - t0) / smallest
    if name == "stream":
        state["req"] = 0
    steps = args.steps
    by_time = int(args.ref_seconds / max(steps * est, 1e-9))
    per_step = max(smallest, min(-(-total // steps), by_time))
    secs, units, done = [], 0, 0
    for k in range(steps):
        t0 = time.perf_counter()
        got = run(done, per_step)
        secs.append(time.perf_counter() - t0)
        done += got
        units += got * unit_work
    tot = sum(secs)
    cores = int(os.environ.get("OMP_NUM_THREADS", os.cpu_count() or 1))
    what = {"gemm": "share-GEMM rows", "stream": "images of the next request", "conv": "images of the batch"}.get(
        kind, "images")
    covered = "the whole batch once" if done >= total else f"{done} of {total}"
    return {"value": units / tot, "ms_per_step": 1e3 * tot / steps, "units": units,
            "cpu_baseline": {"value": units / tot, "unit": w.get("unit", "img/s"), "cores": cores, "kind": "port",
                             "sample": f"{steps} timed steps of {per_step} {what} each ({covered}, {tot:.1f} s), "
                                       f"after {max(1, args.warmup)} warm-up steps of {smallest}; same inputs "
                                       "and weights as the GPU arm"}}


def line_config(args, w, world):
    """The `config` of both arms' JSON lines (the same dict in both)."""
    cfg = {"workload": w["desc"], "global_batch": args.batch * world, "parallelism": "replicas",
           "l2": "GPU arm: 256 MiB write between timed steps; CPU arm: none",
           "graph": "GPU arm: one CUDA graph per step"}
    if w["kind"] == "gemm":
        cfg.update({"global_batch": None, "M": w["M"], "N": w["N"], "K": w["K"], "truncation": w["fp"],
                    "data_size": f"operands {6 * w['M'] * w['K'] * 8 / 1e6:.0f} MB per share tensor, larger than L2"})
    if w["kind"] == "conv":
        g = conv_geometry(args)
        cfg.update({"conv": {k: g[k] for k in ("H", "W", "Din", "Dout", "f", "stride", "pad")}, "truncation": w["fp"],
                    "data_size": f"input shares {48 * g['batch'] * g['H'] * g['W'] * g['Din'] / 1e6:.0f} MB"})
    return cfg


def tensor_rates(pg, dev):
    """Sustained rates of the tensor-core instruction forms on this GPU (pg_tensor_rate)."""
    ctx = pg.Context(dev.index)
    out = {}
    for key, form, iters in (("tcgen05_f16", pg.RATE_TC_F16, 100000), ("tcgen05_f8_e4m3", pg.RATE_TC_F8, 100000),
                             ("mma_sync_s8", pg.RATE_MMA_S8, 20000), ("mma_sync_f16", pg.RATE_MMA_F16, 20000)):
        r = ctx.tensor_rate(form, iters)
        out[key] = round(r["tops"], 1)
    ctx.close()
    out["unit"] = "TOP/s (2 per multiply-add), one launch over every SM"
    out["note"] = "tcgen05.mma kind::i8 is rejected by ptxas for sm_103a: mma.sync s8 is GB300's only INT8 tensor form"
    return out


# ------------------------------------------------------------------ GPU arm

def _as_device_block(torch, dev, ptr, n):
    class _A:
        __cuda_array_interface__ = {"shape": (n,), "typestr": "<i8", "data": (ptr, False), "version": 3}

    return torch.as_tensor(_A(), device=dev)


def run_ours(args, rank, world, local_rank):
    import torch

    import piranha_gb300 as pg

    torch.cuda.set_device(local_rank)
    dev = torch.device("cuda", local_rank)
    stream = torch.cuda.Stream(device=dev)
    batch = args.batch
    kind = WORKLOADS[args.workload]["kind"]
    if kind == "stream":
        wl = make_stream()
        with torch.cuda.stream(stream):
            return bench_stream(args, pg, torch, stream, dev, wl, world), wl
    if kind == "gemm":
        wl = make_gemm()
        with torch.cuda.stream(stream):
            return bench_gemm(args, pg, torch, stream, dev, wl, world), wl
    if kind == "conv":
        wl = make_conv(args)
        with torch.cuda.stream(stream):
            return bench_conv(args, pg, torch, stream, dev, wl, world), wl
    wl = make_workload(args.workload, batch)

    if kind == "fcnet":
        with torch.cuda.stream(stream):
            return bench_fcnet(args, pg, torch, stream, dev, wl, batch, world), wl

    forms = {"u64": [pg.FORM_U64], "tc": [pg.FORM_LIMB_TC], "auto": [pg.FORM_LIMB_TC, pg.FORM_U64]}[args.form]
    fn = bench_form if kind == "infer3" else bench_train
    result = None
    with torch.cuda.stream(stream):
        for form in forms:
            try:
                result = fn(args, pg, torch, stream, dev, form, wl, batch, world)
                break
            except pg.PiranhaError as e:
                if form == forms[-1]:
                    raise
                print(f"[bench] form {form} unavailable: {e}", file=sys.stderr)
        if result and result["form"] == "limb_tc" and not args.no_compare:
            # the same workload on the plain 64-bit integer CUDA-core form, for the limb/u64 ratio
            u = fn(args, pg, torch, stream, dev, pg.FORM_U64, wl, batch, world)
            result["compare_u64"] = {"value": u["value"], "ms_per_step": u["ms_per_step"],
                                     "gemm_tflops_equiv": u["roofline"]["achieved"],
                                     "limb_over_u64": result["value"] / u["value"]}
        if result and args.workload == "vgg16":
            result["tensor_rates"] = tensor_rates(pg, dev)
    return result, wl


def _setup_net(pg, ctx, dev, wl, batch, fp):
    net = pg.Network(ctx, wl["layers"], batch, fp)
    for i, prm in enumerate(wl["params"]):
        if prm is not None:
            net.set_params(i, pg.to_device(prm[0], dev), pg.to_device(prm[1], dev) if prm[1] is not None else None)
    return net


def max_over_ranks(torch, dev, values):
    """Every rank's timings replaced by their maximum over the ranks (the job
    is as slow as its slowest replica)."""
    t = torch.tensor(values, device=dev, dtype=torch.float64)
    torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
    return [float(x) for x in t]


def aggregate(world, units_per_step, steps, seconds):
    """Whole-job throughput: every replica's units over the slowest replica's time."""
    return world * units_per_step * steps / seconds


def _timed(args, torch, stream, dev, world, step, flush, per_step=None):
    """K timed steps with an L2 flush before each (outside the event pair)."""
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    sampler = ClockSampler(dev.index)
    sampler.start()
    wall0 = time.perf_counter()
    step_ms = []
    for k in range(args.steps):
        flush.fill_(k & 0xFF)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        step()
        e1.record(stream)
        stream.synchronize()
        step_ms.append(e0.elapsed_time(e1))
        if per_step:
            per_step()
    torch.cuda.synchronize()
    wall = time.perf_counter() - wall0
    if world > 1:
        torch.distributed.barrier()
    clocks = sampler.stop()
    dev_s = sum(step_ms) / 1e3
    if world > 1:
        dev_s, wall = max_over_ranks(torch, dev, [dev_s, wall])
    return dev_s, wall, clocks


def _e2e(args, torch, stream, dev, world, step, flush):
    for _ in range(max(1, args.warmup)):
        step()
    stream.synchronize()
    ms = []
    for k in range(args.steps):
        flush.fill_(k & 0xFF)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        step()
        e1.record(stream)
        stream.synchronize()
        ms.append(e0.elapsed_time(e1))
    s = sum(ms) / 1e3
    if world > 1:
        (s,) = max_over_ranks(torch, dev, [s])
    return s


def bench_form(args, pg, torch, stream, dev, form, wl, batch, world):
    """Secure inference through the network executor (one CUDA graph per forward)."""
    fp = WORKLOADS[args.workload]["fp"]
    layers = wl["layers"]
    macs = ring_macs(layers, batch)
    ctx = pg.Context(dev.index, stream=stream, form=form)
    ctx.set_autotune(not args.no_autotune)
    net = _setup_net(pg, ctx, dev, wl, batch, fp)
    net.enable_timing(True)
    net.capture()
    xin = pg.to_device(wl["x"], dev).reshape(-1)
    _as_device_block(torch, dev, net.input_buffers()[0], 6 * net.in_n).copy_(xin)
    flush = torch.empty(256 << 20, dtype=torch.uint8, device=dev)
    stream.synchronize()
    for _ in range(args.warmup):
        net.forward_resident()
    stream.synchronize()

    layer_ms = np.zeros(len(layers))

    def acc_layers():
        layer_ms[:] += np.array(net.layer_times_ms())

    launches0 = ctx.kernel_launches()
    comm0 = ctx.comm()
    dev_s, wall, clocks = _timed(args, torch, stream, dev, world, net.forward_resident, flush, acc_layers)
    launches = ctx.kernel_launches() - launches0
    comm1 = ctx.comm()
    value = aggregate(world, batch, args.steps, dev_s)

    # dominant kernel: the fused share-GEMM of the conv layers (FC layers when there are none)
    gemm_idx = sorted(i for i in macs if layers[i][0] == "cnn") or sorted(macs)
    gemm_ms = float(sum(layer_ms[i] for i in gemm_idx)) / args.steps
    gemm_macs = sum(macs[i] for i in gemm_idx)
    achieved = gemm_macs * LIMB_FLOPS_PER_RING_MAC / (gemm_ms / 1e3) / 1e12
    plans = [net.layer_plan(i) for i in range(len(layers))]
    exe = executed_ring_macs(layers, batch, [p["form"] == 1 and p["posmajor"] for p in plans])
    exe_macs = sum(exe[i] for i in gemm_idx)
    executed = exe_macs * LIMB_FLOPS_PER_RING_MAC / (gemm_ms / 1e3) / 1e12
    peaks = load_peaks()
    peak = peaks.get("bf16_tflops", 1900.0)
    peak_note = "of measured" if "bf16_tflops" in peaks else "of fallback"
    what = (f"share-GEMM implicit conv (all {len(gemm_idx)} convs)" if layers[gemm_idx[0]][0] == "cnn"
            else f"share-GEMM FC layers ({len(gemm_idx)})")

    in_host = torch.empty(6 * net.in_n, dtype=torch.int64, pin_memory=True)
    in_host.copy_(xin.cpu())
    out_host = torch.empty(6 * net.out_n, dtype=torch.int64, pin_memory=True)
    e2e_s = _e2e(args, torch, stream, dev, world, lambda: net.forward_host(in_host.data_ptr(), out_host.data_ptr()),
                 flush)

    traffic = None
    if args.workload == "vgg16" and batch == BATCH and form == pg.FORM_LIMB_TC:
        traffic = VGG16_B128_LIMB_TRAFFIC
    out = {
        "form": "limb_tc" if form == pg.FORM_LIMB_TC else "u64",
        "value": value,
        "ms_per_step": 1e3 * dev_s / args.steps,
        "wall_s": wall,
        "e2e": {"value": aggregate(world, batch, args.steps, e2e_s), "unit": "img/s",
                "h2d_bytes_per_step": 6 * net.in_n * 8, "d2h_bytes_per_step": 6 * net.out_n * 8},
        "gpu_launches": int(launches),
        "clocks": clocks,
        "roofline": {"bound": "tensor", "achieved": achieved, "peak": peak, "unit": "TFLOP/s",
                     "frac": achieved / peak, "traffic": traffic,
                     "traffic_unit": "DRAM bytes per forward over the conv launches (ncu)" if traffic else None,
                     "kernel": what,
                     "work": f"{LIMB_FLOPS_PER_RING_MAC} limb-tensor flops per ring MAC, {gemm_macs:.4g} ring MACs/forward "
                             "(dense convolutions, zero-padding taps included, as the reference's convolution "
                             "defines the work)",
                     "executed": {"achieved": executed, "frac": executed / peak, "ring_macs": exe_macs,
                                  "note": "the tensor flops the kernels run: the small layers' position-major tiles "
                                          "skip the zero-padding taps"},
                     "peak_source": f"bf16_tflops {peak_note}"},
        "comm_per_party_per_step": {"tx_bytes": int((comm1["tx"][0] - comm0["tx"][0]) // args.steps),
                                    "rounds": int((comm1["rounds"] - comm0["rounds"]) // args.steps)},
        "layer_ms": [round(float(v) / args.steps, 4) for v in layer_ms],
        "layer_plans": ["" if p["form"] == 0 else "u64" if p["form"] == 2 else
                        ("pos" if p["posmajor"] else "rect") + f"/split{p['split']}" for p in plans],
    }
    net.close()
    ctx.close()
    return out


def bench_train(args, pg, torch, stream, dev, form, wl, batch, world):
    """One SGD iteration (forward + revealed-softmax backward + updates) per step, one CUDA graph."""
    w = WORKLOADS[args.workload]
    fp, lr = w["fp"], w["log_lr"]
    layers = wl["layers"]
    macs = ring_macs(layers, batch)
    ctx = pg.Context(dev.index, stream=stream, form=form)
    ctx.set_autotune(not args.no_autotune)
    net = _setup_net(pg, ctx, dev, wl, batch, fp)
    xin = pg.to_device(wl["x"], dev).reshape(-1)
    lin = pg.to_device(wl["labels"], dev).reshape(-1)
    _as_device_block(torch, dev, net.input_buffers()[0], 6 * net.in_n).copy_(xin)
    _as_device_block(torch, dev, net.label_buffers()[0], 6 * net.out_n).copy_(lin)
    stream.synchronize()
    net.capture_train(lr)
    flush = torch.empty(256 << 20, dtype=torch.uint8, device=dev)
    for _ in range(args.warmup):
        net.train_resident()
    stream.synchronize()
    launches0 = ctx.kernel_launches()
    comm0 = ctx.comm()
    dev_s, wall, clocks = _timed(args, torch, stream, dev, world, net.train_resident, flush)
    launches = ctx.kernel_launches() - launches0
    comm1 = ctx.comm()
    value = aggregate(world, batch, args.steps, dev_s)
    # forward share-GEMMs plus the backward's two per layer (input gradient, weight gradient)
    total_macs = 3 * sum(macs.values())
    achieved = total_macs * LIMB_FLOPS_PER_RING_MAC / (dev_s / args.steps) / 1e12
    peaks = load_peaks()
    peak = peaks.get("bf16_tflops_sustained", peaks.get("bf16_tflops", 1700.0))
    peak_note = "of measured" if peaks else "of fallback"

    in_host = torch.empty(6 * net.in_n, dtype=torch.int64, pin_memory=True)
    in_host.copy_(xin.cpu())
    lab_host = torch.empty(6 * net.out_n, dtype=torch.int64, pin_memory=True)
    lab_host.copy_(lin.cpu())
    out_host = torch.empty(6 * net.out_n, dtype=torch.int64, pin_memory=True)
    e2e_s = _e2e(args, torch, stream, dev, world,
                 lambda: net.train_host(in_host.data_ptr(), lab_host.data_ptr(), out_host.data_ptr(), lr), flush)
    out = {
        "form": "limb_tc" if form == pg.FORM_LIMB_TC else "u64",
        "value": value,
        "ms_per_step": 1e3 * dev_s / args.steps,
        "wall_s": wall,
        "e2e": {"value": aggregate(world, batch, args.steps, e2e_s), "unit": "img/s",
                "h2d_bytes_per_step": 6 * (net.in_n + net.out_n) * 8, "d2h_bytes_per_step": 6 * net.out_n * 8},
        "gpu_launches": int(launches),
        "clocks": clocks,
        "roofline": {"bound": "tensor", "achieved": achieved, "peak": peak, "unit": "TFLOP/s",
                     "frac": achieved / peak, "traffic": None,
                     "kernel": "whole training step (share-GEMMs of forward, input and weight gradients)",
                     "work": f"{LIMB_FLOPS_PER_RING_MAC} limb-tensor flops per ring MAC, {total_macs:.4g} ring MACs/step; "
                             "time includes every non-GEMM launch, so frac is a lower bound",
                     "peak_source": f"bf16_tflops_sustained {peak_note}"},
        "comm_per_party_per_step": {"tx_bytes": int((comm1["tx"][0] - comm0["tx"][0]) // args.steps),
                                    "rounds": int((comm1["rounds"] - comm0["rounds"]) // args.steps)},
    }
    net.close()
    ctx.close()
    return out


def _gemm_form(args, pg, torch, stream, dev, form, A, B, M, N, K, world, steps, warmup, e2e_host=None, op=None):
    """One form of the share-GEMM (or of `op(ctx, A, B, C)` with an M x N
    output): eager call (sizes the scratch), one captured graph, warm-up and
    timed replays; optionally the end-to-end replays."""
    fp = WORKLOADS["gemm"]["fp"]
    if op is None:
        def op(ctx, a, b, c):
            pg.matmul(ctx, a, b, c, M, N, K, 1, 1, 1, fp)
    ctx = pg.Context(dev.index, stream=stream, form=form)
    ctx.set_autotune(not args.no_autotune)
    C = pg.empty_shares(M * N, device=dev)
    op(ctx, A, B, C)
    with ctx.capture() as graph:
        op(ctx, A, B, C)
    for _ in range(warmup):
        graph.launch()
    stream.synchronize()
    flush = torch.empty(256 << 20, dtype=torch.uint8, device=dev)
    sub_args = argparse.Namespace(**{**vars(args), "steps": steps})
    launches0, comm0 = ctx.kernel_launches(), ctx.comm()
    dev_s, wall, clocks = _timed(sub_args, torch, stream, dev, world, graph.launch, flush)
    res = {"dev_s": dev_s, "wall": wall, "clocks": clocks, "launches": ctx.kernel_launches() - launches0,
           "comm0": comm0, "comm1": ctx.comm()}
    if e2e_host is not None:
        # End to end, pipelined over two buffer sets: step k's operands go up
        # on one copy stream while step k-1 computes, and its result comes
        # back on another while step k+1 computes. Every step's host copies
        # are inside the timed region (first upload to last download).
        a_h, b_h, c_h = e2e_host
        A2, B2 = A.clone(), B.clone()
        C2 = pg.empty_shares(M * N, device=dev)
        op(ctx, A2, B2, C2)
        with ctx.capture() as graph2:
            op(ctx, A2, B2, C2)
        sets = [(A, B, C, graph), (A2, B2, C2, graph2)]
        up, down = torch.cuda.Stream(device=dev), torch.cuda.Stream(device=dev)

        def run(n):
            t0, t1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            h2d = [torch.cuda.Event() for _ in range(n)]
            comp = [torch.cuda.Event() for _ in range(n)]
            d2h = [torch.cuda.Event() for _ in range(n)]
            t0.record(up)
            for k in range(n):
                a, b, c, gr = sets[k % 2]
                if k >= 2:
                    up.wait_event(comp[k - 2])  # the set's previous step has read its operands
                with torch.cuda.stream(up):
                    a.copy_(a_h, non_blocking=True)
                    b.copy_(b_h, non_blocking=True)
                h2d[k].record(up)
                stream.wait_event(h2d[k])
                if k >= 2:
                    stream.wait_event(d2h[k - 2])  # the set's previous result is downloaded
                gr.launch()
                comp[k].record(stream)
                down.wait_event(comp[k])
                with torch.cuda.stream(down):
                    c_h.copy_(c, non_blocking=True)
                d2h[k].record(down)
            t1.record(down)
            for st in (up, stream, down):
                st.synchronize()
            return t0.elapsed_time(t1) / 1e3

        run(max(2, warmup))
        e2e_s = run(steps)
        if world > 1:
            (e2e_s,) = max_over_ranks(torch, dev, [e2e_s])
        res["e2e_s"] = e2e_s
        graph2.close()
        del A2, B2, C2
    graph.close()
    del C
    ctx.close()
    return res


def bench_gemm(args, pg, torch, stream, dev, wl, world):
    """3PC share-GEMM microbenchmark: pg.matmul (localMatMul over the concatenated K, dividePublic3out3 with
    its reshare) at M = N = K = 4096, replayed from one CUDA graph; the limb tensor-core form, with the plain
    u64 form beside it."""
    M, N, K = wl["M"], wl["N"], wl["K"]
    A = pg.to_device(wl["A"], dev)
    B = pg.to_device(wl["B"], dev)
    macs = 6 * M * N * K
    a_h = torch.empty(A.shape, dtype=A.dtype, pin_memory=True)
    b_h = torch.empty(B.shape, dtype=B.dtype, pin_memory=True)
    a_h.copy_(A.cpu())
    b_h.copy_(B.cpu())
    c_h = torch.empty((3, 2, M * N), dtype=torch.int64, pin_memory=True)
    form = pg.FORM_U64 if args.form == "u64" else pg.FORM_LIMB_TC
    r = _gemm_form(args, pg, torch, stream, dev, form, A, B, M, N, K, world, args.steps, args.warmup,
                   (a_h, b_h, c_h))
    peaks = load_peaks()
    peak = peaks.get("bf16_tflops")
    achieved = LIMB_FLOPS_PER_RING_MAC * macs * args.steps / r["dev_s"] / 1e12
    out = {
        "form": "limb_tc" if form == pg.FORM_LIMB_TC else "u64",
        "unit": "ring-MAC/s",
        "value": aggregate(world, macs, args.steps, r["dev_s"]),
        "ms_per_step": 1e3 * r["dev_s"] / args.steps,
        "wall_s": r["wall"],
        "e2e": {"value": aggregate(world, macs, args.steps, r["e2e_s"]), "unit": "ring-MAC/s", "pipelined": True,
                "h2d_bytes_per_step": int(A.numel() + B.numel()) * 8, "d2h_bytes_per_step": int(c_h.numel()) * 8},
        "gpu_launches": int(r["launches"]),
        "clocks": r["clocks"],
        "roofline": {"bound": "tensor", "achieved": achieved, "peak": peak, "unit": "TFLOP/s",
                     "frac": achieved / peak if peak else None, "traffic": None,
                     "kernel": "share-GEMM (limb_tma_kernel with its operand image and packing launches)",
                     "work": f"72 limb-tensor flops per ring MAC, {macs:.4g} ring MACs/step; the time includes "
                             "the image and pack launches, so frac is a lower bound for the GEMM kernel",
                     "peak_source": "bf16_tflops of measured" if peak else None},
        "comm_per_party_per_step": {"tx_bytes": int((r["comm1"]["tx"][0] - r["comm0"]["tx"][0]) // args.steps),
                                    "rounds": int((r["comm1"]["rounds"] - r["comm0"]["rounds"]) // args.steps)},
    }
    if form == pg.FORM_LIMB_TC and not args.no_compare:
        u = _gemm_form(args, pg, torch, stream, dev, pg.FORM_U64, A, B, M, N, K, world, max(2, args.steps // 4), 1)
        uv = macs * max(2, args.steps // 4) / u["dev_s"]
        out["compare_u64"] = {"value": uv, "ms_per_step": 1e3 * u["dev_s"] / max(2, args.steps // 4),
                              "gemm_tflops_equiv": LIMB_FLOPS_PER_RING_MAC * uv / 1e12,
                              "limb_over_u64": out["value"] / world / uv}
    if args.sweep:
        sweep = []
        shapes = [(n, n, n) for n in (512, 1024, 2048, 4096, 8192)] + [
            (1024, 8192, 2048), (8192, 512, 4096), (2048, 2048, 8192), (8192, 8192, 512), (512, 4096, 8192)]
        for sM, sN, sK in shapes:
            As = torch.randint(-2**63, 2**63 - 1, (3, 2, sM * sK), dtype=torch.int64, device=dev)
            Bs = torch.randint(-2**63, 2**63 - 1, (3, 2, sK * sN), dtype=torch.int64, device=dev)
            row = {"M": sM, "N": sN, "K": sK}
            work = 6 * sM * sN * sK
            for name, fm in (("limb_tc", pg.FORM_LIMB_TC), ("u64", pg.FORM_U64)):
                st = 3 if work <= 6 * 4096 ** 3 or name == "limb_tc" else 2
                rr = _gemm_form(args, pg, torch, stream, dev, fm, As, Bs, sM, sN, sK, 1, st, 1)
                row[name] = work * st / rr["dev_s"]
            row["limb_over_u64"] = row["limb_tc"] / row["u64"]
            row["limb_tflops_equiv"] = LIMB_FLOPS_PER_RING_MAC * row["limb_tc"] / 1e12
            sweep.append(row)
            del As, Bs
        out["sweep"] = sweep
    return out


def bench_conv(args, pg, torch, stream, dev, wl, world):
    """One RSS convolution layer (fprop with truncation by 2^26), replayed from
    one CUDA graph, in the form --form picks (the limb form by default, with
    the u64 form beside it)."""
    g = wl
    X = pg.to_device(g["X"], dev)
    F = pg.to_device(g["F"], dev)
    macs = conv_macs(g)
    n_out = g["batch"] * g["P"] * g["Q"] * g["Dout"]
    x_h = torch.empty(X.shape, dtype=X.dtype, pin_memory=True)
    f_h = torch.empty(F.shape, dtype=F.dtype, pin_memory=True)
    x_h.copy_(X.cpu())
    f_h.copy_(F.cpu())
    c_h = torch.empty((3, 2, n_out), dtype=torch.int64, pin_memory=True)

    def op(ctx, a, b, c):
        pg.convolution(ctx, a, b, c, pg.FPROP, g["batch"], g["H"], g["W"], g["f"], g["Din"], g["Dout"], g["stride"],
                       g["pad"], 26)

    form = pg.FORM_U64 if args.form == "u64" else pg.FORM_LIMB_TC
    r = _gemm_form(args, pg, torch, stream, dev, form, X, F, n_out, 1, 1, world, args.steps, args.warmup,
                   (x_h, f_h, c_h), op=op)
    peaks = load_peaks()
    peak = peaks.get("bf16_tflops")
    achieved = LIMB_FLOPS_PER_RING_MAC * macs * args.steps / r["dev_s"] / 1e12
    out = {
        "form": "limb_tc" if form == pg.FORM_LIMB_TC else "u64",
        "unit": "ring-MAC/s",
        "value": aggregate(world, macs, args.steps, r["dev_s"]),
        "ms_per_step": 1e3 * r["dev_s"] / args.steps,
        "wall_s": r["wall"],
        "e2e": {"value": aggregate(world, macs, args.steps, r["e2e_s"]), "unit": "ring-MAC/s", "pipelined": True,
                "h2d_bytes_per_step": int(X.numel() + F.numel()) * 8, "d2h_bytes_per_step": int(c_h.numel()) * 8},
        "gpu_launches": int(r["launches"]),
        "clocks": r["clocks"],
        "roofline": {"bound": "tensor", "achieved": achieved, "peak": peak, "unit": "TFLOP/s",
                     "frac": achieved / peak if peak else None, "traffic": None,
                     "kernel": "share-conv (the form's GEMM kernel with its operand image, packing and reduce "
                               "launches)",
                     "work": f"72 limb-tensor flops per ring MAC, {macs:.4g} ring MACs/step",
                     "peak_source": "bf16_tflops of measured" if peak else None},
        "comm_per_party_per_step": {"tx_bytes": int((r["comm1"]["tx"][0] - r["comm0"]["tx"][0]) // args.steps),
                                    "rounds": int((r["comm1"]["rounds"] - r["comm0"]["rounds"]) // args.steps)},
    }
    if form == pg.FORM_LIMB_TC and not args.no_compare:
        st = max(2, args.steps // 4)
        u = _gemm_form(args, pg, torch, stream, dev, pg.FORM_U64, X, F, n_out, 1, 1, world, st, 1, op=op)
        uv = macs * st / u["dev_s"]
        out["compare_u64"] = {"value": uv, "ms_per_step": 1e3 * u["dev_s"] / st,
                              "gemm_tflops_equiv": LIMB_FLOPS_PER_RING_MAC * uv / 1e12,
                              "limb_over_u64": out["value"] / world / uv}
    return out


def bench_fcnet(args, pg, torch, stream, dev, wl, batch, world):
    """2PC / 4PC FC net: FCLayer::forward + ReLU per layer through the TPC / FPC entry points, captured as one
    CUDA graph (ctx.capture) after an eager forward."""
    w = WORKLOADS[args.workload]
    fp, ring = w["fp"], w["ring"]
    proto = pg.tpc if w["parties"] == 2 else pg.fpc
    layers = wl["layers"]
    ctx = pg.Context(dev.index, stream=stream)
    tdt = torch.int32 if ring == "u32" else torch.int64

    def dev_t(a):
        return torch.from_numpy(np.ascontiguousarray(a).view(np.int32 if ring == "u32" else np.int64)).to(dev)

    x = dev_t(wl["x"])
    prm = [None if p is None else (dev_t(p[0]), dev_t(p[1])) for p in wl["params"]]
    bufs = []
    for L in layers:
        n = batch * (L[2] if L[0] == "fc" else L[1])
        bufs.append((proto.empty(n, ring, dev), proto.zeros(n, "u8", dev) if L[0] == "relu" else None))

    def forward(inp):
        cur = inp
        for L, p, (o, d) in zip(layers, prm, bufs):
            if L[0] == "fc":
                proto.fc_forward(ctx, cur, p[0], p[1], o, batch, L[1], L[2], fp)
            else:
                proto.ReLU(ctx, cur, o, d)
            cur = o
        return cur

    flush = torch.empty(256 << 20, dtype=torch.uint8, device=dev)
    # one eager forward sizes the context scratch, then the whole forward is one graph
    forward(x)
    with ctx.capture() as graph:
        y = forward(x)
    for _ in range(args.warmup):
        graph.launch()
    stream.synchronize()
    launches0 = ctx.kernel_launches()
    comm0 = ctx.comm(w["parties"])
    dev_s, wall, clocks = _timed(args, torch, stream, dev, world, graph.launch, flush)
    launches = ctx.kernel_launches() - launches0
    comm1 = ctx.comm(w["parties"])
    value = aggregate(world, batch, args.steps, dev_s)
    macs = sum(batch * L[1] * L[2] for L in layers if L[0] == "fc")

    x_host = torch.empty(x.shape, dtype=tdt, pin_memory=True)
    x_host.copy_(x.cpu())
    y_host = torch.empty(bufs[-1][0].shape, dtype=tdt, pin_memory=True)

    def e2e_step():
        x.copy_(x_host, non_blocking=True)
        graph.launch()
        y_host.copy_(y, non_blocking=True)

    e2e_s = _e2e(args, torch, stream, dev, world, e2e_step, flush)
    elt = 4 if ring == "u32" else 8
    out = {
        "form": "tpc" if w["parties"] == 2 else "fpc",
        "value": value,
        "ms_per_step": 1e3 * dev_s / args.steps,
        "wall_s": wall,
        "e2e": {"value": aggregate(world, batch, args.steps, e2e_s), "unit": "img/s",
                "h2d_bytes_per_step": int(x.numel()) * elt, "d2h_bytes_per_step": int(bufs[-1][0].numel()) * elt},
        "gpu_launches": int(launches),
        "clocks": clocks,
        "roofline": {"bound": "launch", "achieved": None, "peak": None, "unit": None, "frac": None, "traffic": None,
                     "kernel": "per-layer protocol launches in one graph",
                     "work": f"{macs:.4g} plaintext MACs per forward in {len(layers)} layers: far too little to "
                             "load the tensor cores or HBM, so the step is launch-bound"},
        "comm_per_party_per_step": {"tx_bytes": [int((a - b) // args.steps) for a, b in zip(comm1["tx"], comm0["tx"])],
                                    "rounds": int((comm1["rounds"] - comm0["rounds"]) // args.steps)},
    }
    graph.close()
    ctx.close()
    return out


def bench_stream(args, pg, torch, stream, dev, wl, world):
    """The request stream, served in arrival order on one stream by
    piranha_gb300.stream: waiting requests of the same model are packed into
    one replay of a captured network whose batch bucket holds them: the
    smallest such bucket, or a larger bucket of the same model whose replay
    timed faster (the oldest waiting request opens a pack, the next 16 waiting
    requests of its model join it while it stays within 128 images; --no-pack
    serves each request alone). A pack's latency is its CUDA-event time from
    the start of its input copies to the end of its output copies; every
    request of a pack has that latency. The stream runs args.warmup times
    untimed, then once timed per pass: a device-resident pass (inputs staged
    in HBM beforehand) and an end-to-end pass (pinned host shares in and out),
    each pack alone on the stream; the end-to-end throughput comes from a
    third, pipelined pass in which the next pack's input copies overlap the
    current forward."""
    from piranha_gb300 import stream as st

    models, params, reqs = wl
    fp = WORKLOADS["stream"]["fp"]
    form = pg.FORM_U64 if args.form == "u64" else pg.FORM_LIMB_TC
    ctx = pg.Context(dev.index, stream=stream, form=form)
    ctx.set_autotune(not args.no_autotune)
    server = st.StreamServer(pg, ctx, {m: (models[m], params[m]) for m in models}, fp, dev)
    packs = st.plan_packs([(m, b) for m, b, _ in reqs], cap=128, lookahead=0 if args.no_pack else 16)
    for p in packs:
        server.network(p.model, p.bucket)
    stream.synchronize()
    moved = 0
    if not args.no_autotune:
        tuned = server.tune_buckets(packs)
        moved = sum(a.bucket != b.bucket for a, b in zip(packs, tuned))
        packs = tuned

    per_img_out = 10
    dev_in = [torch.from_numpy(np.ascontiguousarray(x).reshape(6, -1).view(np.int64)).to(dev) for _, _, x in reqs]
    host_in = [t.cpu().pin_memory() for t in dev_in]
    dev_out = [torch.empty((6, b * per_img_out), dtype=torch.int64, device=dev) for _, b, _ in reqs]
    host_out = [torch.empty((6, b * per_img_out), dtype=torch.int64, pin_memory=True) for _, b, _ in reqs]

    def serve(resident):
        evs = []
        for p in packs:
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            server.serve(p, dev_in if resident else host_in, dev_out if resident else host_out)
            e1.record(stream)
            evs.append((p, e0, e1))
        stream.synchronize()
        lat = []
        for p, e0, e1 in evs:
            lat += [e0.elapsed_time(e1)] * len(p.requests)
        return lat, sum(e0.elapsed_time(e1) for _, e0, e1 in evs) / 1e3

    copy_stream = torch.cuda.Stream(device=dev)
    staged = {}

    def serve_pipelined():
        """End-to-end throughput: the next pack's host-to-device copies run on a
        second stream (into staging buffers) while the current pack computes;
        returns the seconds from the first copy to the last output copy."""
        t0, t1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        copied = [torch.cuda.Event() for _ in packs]
        started = [torch.cuda.Event() for _ in packs]
        t0.record(copy_stream)

        def h2d(k):
            if k > 0:
                copy_stream.wait_event(started[k - 1])
            with torch.cuda.stream(copy_stream):
                for r in packs[k].requests:
                    dev_in[r].copy_(host_in[r], non_blocking=True)
            copied[k].record(copy_stream)

        h2d(0)
        for k, p in enumerate(packs):
            stream.wait_event(copied[k])
            started[k].record(stream)
            if k + 1 < len(packs):
                h2d(k + 1)
            server.serve(p, dev_in, host_out)
        t1.record(stream)
        stream.synchronize()
        copy_stream.synchronize()
        return t0.elapsed_time(t1) / 1e3

    for _ in range(max(1, args.warmup)):
        serve(True)
    launches0 = ctx.kernel_launches()
    sampler = ClockSampler(dev.index)
    sampler.start()
    wall0 = time.perf_counter()
    lat_res, dev_s = serve(True)
    wall = time.perf_counter() - wall0
    clocks = sampler.stop()
    launches = ctx.kernel_launches() - launches0
    lat_e2e, _ = serve(False)
    serve_pipelined()
    e2e_s = serve_pipelined()
    imgs = sum(b for _, b, _ in reqs)
    pct = lambda v, q: float(np.percentile(np.array(v), q))  # noqa: E731
    out = {
        "form": "limb_tc" if form == pg.FORM_LIMB_TC else "u64",
        "value": aggregate(world, imgs, 1, dev_s),
        "ms_per_step": 1e3 * dev_s / len(packs),
        "wall_s": wall,
        "e2e": {"value": aggregate(world, imgs, 1, e2e_s), "unit": "img/s",
                "h2d_bytes_per_step": int(sum(t.numel() * 8 for t in host_in) / len(packs)),
                "d2h_bytes_per_step": int(sum(t.numel() * 8 for t in host_out) / len(packs))},
        "latency_ms": {"resident": {"p50": pct(lat_res, 50), "p99": pct(lat_res, 99), "max": max(lat_res)},
                       "e2e": {"p50": pct(lat_e2e, 50), "p99": pct(lat_e2e, 99), "max": max(lat_e2e)},
                       "note": "per request: its pack's time alone on the stream (input copies to output copies); "
                               "the e2e throughput overlaps the next pack's input copies with the current forward"},
        "requests": len(reqs), "images": imgs, "replays": len(packs),
        "packing": "none (one request per replay)" if args.no_pack else
                   "same-model requests within the next 16 waiting ones, up to 128 images per replay",
        "gpu_launches": int(launches),
        "clocks": clocks,
        "roofline": {"bound": "tensor", "achieved": None, "peak": None, "unit": "TFLOP/s", "frac": None,
                     "traffic": None, "kernel": "see the vgg16 and secureml workloads",
                     "work": "mixed request sizes; the per-model lines carry the kernel fractions"},
        "comm_per_party_per_step": None,
        "networks": sorted(f"{m}@{b}" for m, b in server.nets),
        "bucket_choice": {"moved_to_a_larger_bucket": int(moved),
                          "replay_ms": {f"{m}@{b}": round(1e3 * t, 4) for (m, b), t in sorted(server.times.items())},
                          "rule": "a pack runs on the fastest timed network of its model that holds it (a larger "
                                  "bucket only when at least 3 % faster); --no-autotune keeps the smallest bucket"},
    }
    server.close()
    ctx.close()
    return out


def main():
    args = parse()
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local_rank = int(os.environ.get("LOCAL_RANK", "0"))
    w = WORKLOADS[args.workload]
    dtype = w["ring"]

    if args.impl == "reference":
        if rank != 0:
            return
        wl = (make_stream() if w["kind"] == "stream" else make_gemm() if w["kind"] == "gemm"
              else make_conv(args) if w["kind"] == "conv" else make_workload(args.workload, args.batch))
        r = reference_arm(args, args.workload, wl)
        unit = w.get("unit", "img/s")
        line = {"metric": w["metric"], "value": r["value"], "unit": unit, "impl": "reference", "n_gpus": args.gpus,
                "steps": args.steps, "warmup": args.warmup, "ms_per_step": r["ms_per_step"],
                "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": dtype,
                "data": "synthetic", "config": line_config(args, w, 1),
                "cpu_baseline": r["cpu_baseline"], "e2e": {"value": r["value"], "unit": unit,
                                                           "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
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
        cb = cpu_baseline(args.workload, wl, args.batch, args.cpu_seconds)
    line = {
        "metric": w["metric"], "value": res["value"], "unit": res.get("unit", "img/s"), "n_gpus": world,
        "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": res["ms_per_step"], "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": dtype, "data": "synthetic",
        "config": line_config(args, w, world), "form": res["form"],
        "e2e": res["e2e"], "gpu_launches": res["gpu_launches"], "clocks": res["clocks"],
        "roofline": res["roofline"], "cpu_baseline": cb,
        "comm_per_party_per_step": res["comm_per_party_per_step"],
    }
    if "layer_ms" in res:
        line["layer_ms"] = res["layer_ms"]
    if "layer_plans" in res:
        line["layer_plans"] = res["layer_plans"]
    for k in ("latency_ms", "requests", "images", "replays", "packing", "networks", "bucket_choice", "sweep"):
        if k in res:
            line[k] = res[k]
    if "compare_u64" in res:
        line["compare_u64_form"] = res["compare_u64"]
    if "tensor_rates" in res:
        line["tensor_rates"] = res["tensor_rates"]
    print(json.dumps(line))


if __name__ == "__main__":
    main()
