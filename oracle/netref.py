"""Layer-by-layer oracle composition of NeuralNetwork::forward and ::backward
(NeuralNetwork.cu:109-148, :439-460).

Used by the network parity tests and the CPU-baseline leg of bench.py: the
same layer tuples as piranha_gb300.Network, evaluated with the CPU oracle.
"""
import numpy as np

import oracle as orc


def fc_forward(x, w, b, batch, din, dout, fp=26):
    act = orc.matmul(x, w, batch, dout, din, 1, 1, 1, fp)
    if b is not None:
        for p in range(3):
            for s in range(2):
                act[p, s] = orc.element_vector_add(act[p, s], b[p, s], False, dout, batch)
    return act


def forward(layers, params, x, batch, fp=26, comm=None, keep=False, bits=None):
    """params[i] = (w, b) views (or None); returns the output (and every layer's output if keep).
    bits, a list, receives each layer's derivative bits (reluPrime / maxPrime, None for FC / CNN)."""
    outs = []
    for L, prm in zip(layers, params):
        kind = L[0]
        d = None
        if kind == "fc":
            x = fc_forward(x, prm[0], prm[1], batch, L[1], L[2], fp)
            if comm is not None:
                n = batch * L[2]
                comm.buf[0:3] += np.uint64(2 * n * 8)
                comm.buf[4:7] += np.uint64(2 * n * 8)
                comm.buf[8] += np.uint64(1)
        elif kind == "cnn":
            H, W, Din, Dout, f, s, pd = L[1:]
            x = orc.convolution(x, prm[0], orc.FPROP, batch, H, W, f, Din, Dout, s, pd, fp, comm)
        elif kind == "relu":
            x, d = orc.relu(x, comm=comm)
        elif kind == "maxpool":
            H, W, C, pool, stride = L[1:]
            x, d = orc.maxpool_layer(x, H, W, C, pool, stride, batch, fp, comm=comm)
        elif kind == "avgpool":
            H, W, C, pool, stride = L[1:]
            x = orc.avgpool_layer(x, H, W, C, pool, stride, batch, comm=comm)
        else:
            raise ValueError(kind)
        if keep:
            outs.append(x)
        if bits is not None:
            bits.append(d)
    return (x, outs) if keep else x


def backward(layers, params, x, outs, bits, labels, batch, fp=26, log_lr=5, comm=None):
    """NeuralNetwork::backward (NeuralNetwork.cu:136-148, :439-460): the revealed
    softmax gradient of the last activation, then every layer's backward from
    the last to the first. Returns (updated params, each layer's deltas)."""
    params = [None if p is None else (p[0].copy(), None if p[1] is None else p[1].copy()) for p in params]
    deltas = [None] * len(layers)
    delta = orc.reveal_softmax_grad(outs[-1], labels, batch, fp, comm)
    for i in range(len(layers) - 1, -1, -1):
        L = layers[i]
        fwd_in = outs[i - 1] if i > 0 else x
        kind = L[0]
        if kind == "fc":
            d, w, b = orc.fc_layer_backward(delta, fwd_in, params[i][0], params[i][1], batch, L[1], L[2], fp, log_lr,
                                            comm)
            params[i] = (w, b)
        elif kind == "cnn":
            H, W, Din, Dout, f, s, pd = L[1:]
            d, w = orc.cnn_layer_backward(delta, fwd_in, params[i][0], batch, H, W, Din, Dout, f, s, pd, fp, log_lr,
                                          comm)
            params[i] = (w, None)
        elif kind == "relu":
            d = orc.relu_layer_backward(delta, bits[i], comm)
        elif kind == "maxpool":
            H, W, C, pool, stride = L[1:]
            d = orc.maxpool_layer_backward(delta, bits[i], H, W, C, pool, stride, batch, comm)
        elif kind == "avgpool":
            H, W, C, pool, stride = L[1:]
            d = orc.avgpool_layer_backward(delta, H, W, C, pool, batch, comm)
        else:
            raise ValueError(kind)
        deltas[i] = d
        delta = d
    return params, deltas


def train_step(layers, params, x, labels, batch, fp=26, log_lr=5, comm=None):
    """One forward + backward + SGD update (main.cu:314-330 for one iteration)."""
    bits = []
    out, outs = forward(layers, params, x, batch, fp, comm, keep=True, bits=bits)
    new_params, deltas = backward(layers, params, x, outs, bits, labels, batch, fp, log_lr, comm)
    return out, outs, new_params, deltas


def vgg16_layers(maxpool=True):
    """VGG16 of files/models/vgg16-cifar10.json; maxpool=True replaces each averagepool by a 2x2/2 maxpool."""
    L = []
    hw, c = 32, 3
    blocks = [(64, 2), (128, 2), (256, 3), (512, 3), (512, 3)]
    for width, reps in blocks:
        for r in range(reps):
            L.append(("cnn", hw, hw, c, width, 3, 1, 1))
            c = width
            if r < reps - 1:
                L.append(("relu", hw * hw * c))
        L.append(("maxpool" if maxpool else "avgpool", hw, hw, c, 2, 2))
        hw //= 2
        L.append(("relu", hw * hw * c))
    L += [("fc", 512, 256), ("relu", 256), ("fc", 256, 256), ("relu", 256), ("fc", 256, 10), ("relu", 10)]
    return L


def secureml_layers():
    return [("fc", 784, 128), ("relu", 128), ("fc", 128, 128), ("relu", 128), ("fc", 128, 10), ("relu", 10)]


def lenet_layers():
    return [("cnn", 28, 28, 1, 20, 5, 1, 0), ("maxpool", 24, 24, 20, 2, 2), ("relu", 2880),
            ("cnn", 12, 12, 20, 50, 5, 1, 0), ("maxpool", 8, 8, 50, 2, 2), ("relu", 800),
            ("fc", 800, 500), ("relu", 500), ("fc", 500, 10), ("relu", 10)]


def kaiming_uniform_params(layers, seed, fp=26):
    """Seeded Kaiming-uniform weights (bound sqrt(6/fan_in)), FC bias 0.01, loaded with setPublic."""
    rng = np.random.default_rng(seed)
    params = []
    for L in layers:
        if L[0] == "fc":
            din, dout = L[1], L[2]
            w = rng.uniform(-1, 1, din * dout) * np.sqrt(6.0 / din)
            params.append((orc.set_public(w, fp=fp), orc.set_public(np.full(dout, 0.01), fp=fp)))
        elif L[0] == "cnn":
            H, W, Din, Dout, f = L[1:6]
            w = rng.uniform(-1, 1, Dout * f * f * Din) * np.sqrt(6.0 / (f * f * Din))
            params.append((orc.set_public(w, fp=fp), None))
        else:
            params.append(None)
    return params
