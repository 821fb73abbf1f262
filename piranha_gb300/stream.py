"""Batched secure-inference serving: requests of uneven batch sizes packed
into replays of captured networks.

The reference serves one batch per call of its inference loop
(src/main.cu:227-258). Here waiting requests of the same model are
concatenated image-wise into one replay of a captured network whose batch is
the smallest bucket that holds them: every layer of the forward works image
by image (FC rows, convolution images, ReLU and maxpool elementwise), so each
request's images give the same result in any rows of any larger batch, and
the rows past the packed requests (an earlier replay's images) do not touch
them.

* ``plan_packs`` is the packing policy: the oldest waiting request opens a
  pack; the next waiting requests of its model within a look-ahead window
  join it while the pack stays within ``cap`` images.
* ``StreamServer`` keeps one captured network per (model, bucket), copies a
  pack's input shares into the first rows of the bucket network's input
  buffers, replays its graph and hands out each request's output rows.
* ``StreamServer.tune_buckets`` times each captured network once and moves a
  pack to a larger bucket of its model when that one replays faster (VGG16
  at 128 images runs position-major convolution tiles, which need a multiple
  of 128 images; at 112 it runs rectangle tiles and takes longer).
"""
from __future__ import annotations

from dataclasses import dataclass

import numpy as np

# batch sizes of the captured networks: at most a third of a replay is padding
BUCKETS = (1, 2, 4, 6, 8, 12, 16, 24, 32, 40, 48, 56, 64, 80, 96, 112, 128)


def bucket_for(b: int, buckets=BUCKETS) -> int:
    for x in buckets:
        if x >= b:
            return x
    raise ValueError(f"batch {b} is above the largest bucket {buckets[-1]}")


@dataclass
class Pack:
    model: str
    requests: list  # request indices, in arrival order
    images: int     # total images
    bucket: int     # batch of the network that serves it


def choose_bucket(times: dict, bucket: int, margin: float = 0.03) -> int:
    """times: {bucket: replay seconds} of one model's captured networks. The
    bucket a pack that fits ``bucket`` is served on: the fastest of ``bucket``
    and the larger timed buckets, a larger one only when it is at least
    ``margin`` faster."""
    best, t_best = bucket, times.get(bucket)
    if t_best is None:
        return bucket
    for b in sorted(times):
        if b > bucket and times[b] < t_best * (1.0 - margin):
            best, t_best = b, times[b]
    return best


def plan_packs(requests, cap: int = 128, lookahead: int = 16, buckets=BUCKETS):
    """requests: a sequence of (model, batch) in arrival order. Returns the
    packs in serving order; every request is in exactly one pack."""
    n = len(requests)
    taken = np.zeros(n, dtype=bool)
    packs = []
    head = 0
    while head < n:
        if taken[head]:
            head += 1
            continue
        m, b = requests[head][0], int(requests[head][1])
        if b > cap:
            raise ValueError(f"request {head} has {b} images, more than a pack's {cap}")
        members, total = [head], b
        taken[head] = True
        seen = 0
        j = head + 1
        while j < n and seen < lookahead and total < cap:
            if not taken[j]:
                seen += 1
                if requests[j][0] == m and total + int(requests[j][1]) <= cap:
                    members.append(j)
                    total += int(requests[j][1])
                    taken[j] = True
            j += 1
        packs.append(Pack(m, members, total, bucket_for(total, buckets)))
        head += 1
    return packs


class StreamServer:
    """One captured network per (model, bucket) on ``ctx``; ``models`` maps a
    model name to (layers, params) with params as for Network.set_params."""

    def __init__(self, pg, ctx, models, fp: int = 26, device=None):
        self.pg = pg
        self.ctx = ctx
        self.models = models
        self.fp = fp
        self.device = device if device is not None else "cuda"
        self.nets = {}
        self.n_in = {m: _input_size(L) for m, (L, _) in models.items()}
        self.n_out = {m: _output_size(L) for m, (L, _) in models.items()}
        self.times = {}  # (model, bucket) -> seconds per replay

    def replay_seconds(self, model: str, bucket: int, reps: int = 3) -> float:
        """Seconds per replay of the (model, bucket) network, timed once on the
        host around ``reps`` replays after one warm-up (the stream synchronised
        on both sides)."""
        import time

        key = (model, bucket)
        if key not in self.times:
            net, _, _ = self.network(model, bucket)
            net.forward_resident()
            self.ctx.sync()
            t0 = time.perf_counter()
            for _ in range(reps):
                net.forward_resident()
            self.ctx.sync()
            self.times[key] = (time.perf_counter() - t0) / reps
        return self.times[key]

    def tune_buckets(self, packs):
        """The packs with each one's bucket replaced by the fastest captured
        bucket of its model that holds it (choose_bucket over the buckets the
        packs already use, so no further network is captured)."""
        used = {}
        for p in packs:
            used.setdefault(p.model, set()).add(p.bucket)
        times = {m: {b: self.replay_seconds(m, b) for b in bs} for m, bs in used.items()}
        return [Pack(p.model, p.requests, p.images, choose_bucket(times[p.model], p.bucket)) for p in packs]

    def network(self, model: str, bucket: int):
        """(net, input view (6, in_n), output view (6, out_n)) of the captured network."""
        key = (model, bucket)
        if key not in self.nets:
            pg = self.pg
            layers, params = self.models[model]
            net = pg.Network(self.ctx, layers, bucket, self.fp)
            for i, prm in enumerate(params):
                if prm is not None:
                    net.set_params(i, pg.to_device(prm[0], self.device),
                                   pg.to_device(prm[1], self.device) if prm[1] is not None else None)
            net.capture()
            optrs, on = net.layer_output_ptrs(len(layers) - 1)
            inb = _device_view(net.input_buffers()[0], 6 * net.in_n, self.device).view(6, net.in_n)
            outb = _device_view(optrs[0], 6 * on, self.device).view(6, on)
            inb.zero_()
            self.nets[key] = (net, inb, outb)
        return self.nets[key]

    def serve(self, pack: Pack, inputs, outputs):
        """Enqueue one pack on the context's stream: inputs[r] (a (6, b_r * n_in)
        int64 tensor, device or pinned host) of each request r of the pack go
        into consecutive image rows, the network replays, and each request's
        output rows go to outputs[r] ((6, b_r * n_out), device or pinned host)."""
        net, inb, outb = self.network(pack.model, pack.bucket)
        n_in, n_out = self.n_in[pack.model], self.n_out[pack.model]
        row = 0
        for r in pack.requests:
            k = inputs[r].shape[1] // n_in
            inb[:, row * n_in:(row + k) * n_in].copy_(inputs[r], non_blocking=True)
            row += k
        net.forward_resident()
        row = 0
        for r in pack.requests:
            k = outputs[r].shape[1] // n_out
            outputs[r].copy_(outb[:, row * n_out:(row + k) * n_out], non_blocking=True)
            row += k

    def close(self):
        for net, _, _ in self.nets.values():
            net.close()
        self.nets = {}


def _device_view(ptr, n, device):
    import torch

    class _A:
        __cuda_array_interface__ = {"shape": (n,), "typestr": "<i8", "data": (ptr, False), "version": 3}

    return torch.as_tensor(_A(), device=device if device is not None else "cuda")


def _input_size(layers):
    L = layers[0]
    if L[0] == "fc":
        return L[1]
    if L[0] == "cnn":
        return L[1] * L[2] * L[3]
    if L[0] == "relu":
        return L[1]
    return L[1] * L[2] * L[3]


def _output_size(layers):
    L = layers[-1]
    if L[0] == "fc":
        return L[2]
    if L[0] == "relu":
        return L[1]
    if L[0] == "cnn":
        H, W, Din, Dout, f, s, p = L[1:]
        return ((H + 2 * p - f) // s + 1) * ((W + 2 * p - f) // s + 1) * Dout
    H, W, C, pool, stride = L[1:]
    return ((H - pool) // stride + 1) * ((W - pool) // stride + 1) * C
