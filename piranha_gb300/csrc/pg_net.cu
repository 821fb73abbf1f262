// pg_net.cu — network executor for secure inference: NeuralNetwork::forward
// (src/nn/NeuralNetwork.cu:109-133) over FC / CNN / ReLU / Maxpool layers
// (FCLayer.cu:78-130, CNNLayer.cu:81-115, ReLULayer.cu:51-88,
// MaxpoolLayer.cu:52-131). All share buffers of all layers are allocated once
// in one device arena at creation; a forward is a fixed sequence of fused
// launches on the context stream, which pg_net_capture records as one CUDA
// graph so that a replay costs one launch.
#include <cstring>
#include <vector>

#include "pg_common.cuh"
#include "pg_limb_tma.cuh"

namespace pg {
template <typename T>
int rss_matmul(Ctx *, const T *const *, const T *const *, T *const *, const T *const *, int, int, int, int, int, int,
               int);
template <typename T>
int rss_conv(Ctx *, const T *const *, const T *const *, T *const *, int, int, int, int, int, int, int, int, int, int);
template <typename T, typename U> int rss_relu(Ctx *, const T *const *, size_t, T *const *, U *const *);
template <typename T, typename U>
int rss_maxpool_layer(Ctx *, const T *const *, T *const *, U *const *, int, int, int, int, int, int, int);
}  // namespace pg

using namespace pg;

struct NetLayer {
    int type;
    int p[7];
    size_t in_n, out_n, w_n, b_n, d_n;  // elements per share buffer (activations include the batch)
    uint64_t *w[6], *b[6], *out[6];
    uint8_t *d[6];
    // limb tensor-core form (FC and CNN layers): plan, split-K, packed weights
    lt::Plan plan;
    int split, cps;
    uint8_t *packB;
};

struct pg_net {
    pg_ctx *ctx;
    int batch, fp;
    std::vector<NetLayer> layers;
    void *arena = nullptr;
    size_t arena_bytes = 0;
    uint64_t *in[6];
    size_t in_n = 0, out_n = 0;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    uint64_t comm_per_fwd[9] = {0};  // accounting of one forward, replayed with the graph
    uint64_t launches_per_fwd = 0;
    std::vector<cudaEvent_t> ev;  // 2 per layer when per-layer timing is on (recorded into graphs too)
    // Buffers of the limb tensor-core form, owned by the network (so that a
    // captured graph never points into the context's growable scratch):
    // packed weights of every FC / CNN layer, one digit-plane image and one
    // split-K partial buffer shared by the layers. Set up by the first
    // limb-form forward, which is always eager (capture runs one first).
    void *limb_arena = nullptr;
    uint8_t *limb_image = nullptr;
    uint64_t *limb_partial = nullptr;
};

// Plans, buffer sizes and weight packing of the limb form.
static int net_limb_setup(pg_net *net) {
    Ctx *c = net->ctx;
    auto al = [](size_t b) { return (b + 255) & ~(size_t)255; };
    size_t image = 0, partial = 0, packs = 0;
    const int sms = c->sm_count > 0 ? c->sm_count : 148;
    for (auto &L : net->layers) {
        int st = PG_OK;
        if (L.type == PG_LAYER_FC) st = lt::plan_gemm(c, L.plan, net->batch, L.p[1], L.p[0], 1, 1, 1);
        else if (L.type == PG_LAYER_CNN)
            st = lt::plan_conv(c, L.plan, net->batch, L.p[0], L.p[1], L.p[4], L.p[2], L.p[3], L.p[5], L.p[6]);
        else continue;
        if (st) return st;
        lt::choose_split(L.plan, sms, L.split, L.cps);
        image = image > L.plan.image_bytes ? image : L.plan.image_bytes;
        const size_t pb = lt::partial_bytes(L.plan, L.split);
        partial = partial > pb ? partial : pb;
        packs += al(L.plan.packB_bytes);
    }
    const size_t bytes = al(image) + al(partial) + packs;
    if (cudaMalloc(&net->limb_arena, bytes) != cudaSuccess) {
        cudaGetLastError();
        net->limb_arena = nullptr;
        return set_error(c, PG_ERR_NO_MEMORY, "limb-form buffers of %zu bytes", bytes);
    }
    uint8_t *ptr = (uint8_t *)net->limb_arena;
    net->limb_image = ptr;
    ptr += al(image);
    net->limb_partial = partial ? (uint64_t *)ptr : nullptr;
    ptr += al(partial);
    for (auto &L : net->layers) {
        if (L.type != PG_LAYER_FC && L.type != PG_LAYER_CNN) continue;
        L.packB = ptr;
        ptr += al(L.plan.packB_bytes);
        int st = lt::run_pack(c, L.plan, (const uint64_t *const *)L.w, L.packB);
        if (st) return st;
    }
    return PG_OK;
}

// One FC / CNN layer in the limb form: digit image of the input, GEMM over
// the packed weights (+ split-K reduction), then the message accounting of
// matmul / convolution (RSS.inl:517-538, :790-802).
static int net_limb_layer(pg_net *net, NetLayer &L, const uint64_t *const *in) {
    Ctx *c = net->ctx;
    int st = lt::run_image(c, L.plan, in, net->limb_image);
    if (st) return st;
    const uint64_t *const *bias = L.b_n ? (const uint64_t *const *)L.b : nullptr;
    st = lt::run_gemm(c, L.plan, net->limb_image, L.packB, L.split > 1 ? net->limb_partial : nullptr, L.split, L.cps,
                      L.out, bias, net->fp);
    if (st) return st;
    const uint64_t n_out = (uint64_t)L.plan.M * L.plan.N;
    comm_msg(c, 2 * n_out * 8, 2 * n_out * 8);
    comm_round(c);
    return PG_OK;
}

// Per-layer timing events: inside a stream capture they must be external
// event nodes so that graph replays record them; outside, a plain record.
static int record_event(Ctx *c, cudaEvent_t e) {
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    PG_CHECK_CUDA(c, cudaStreamIsCapturing(c->stream, &cs));
    if (cs == cudaStreamCaptureStatusActive) PG_CHECK_CUDA(c, cudaEventRecordWithFlags(e, c->stream, cudaEventRecordExternal));
    else PG_CHECK_CUDA(c, cudaEventRecord(e, c->stream));
    return PG_OK;
}

static int net_run(pg_net *net, const uint64_t *const in[6]) {
    Ctx *c = net->ctx;
    const uint64_t *const *cur = in;
    if (c->form == PG_FORM_LIMB_TC && !net->limb_arena) {
        cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
        PG_CHECK_CUDA(c, cudaStreamIsCapturing(c->stream, &cs));
        if (cs != cudaStreamCaptureStatusNone)
            return set_error(c, PG_ERR_INVALID_ARG, "limb-form buffers must be set up by an eager forward first");
        int st = net_limb_setup(net);
        if (st) return st;
    }
    for (size_t li = 0; li < net->layers.size(); li++) {
        NetLayer &L = net->layers[li];
        int st = PG_OK;
        if (!net->ev.empty() && (st = record_event(c, net->ev[2 * li]))) return st;
        switch (L.type) {
            case PG_LAYER_FC: {
                const uint64_t *const *bias = L.b_n ? (const uint64_t *const *)L.b : nullptr;
                st = c->form == PG_FORM_LIMB_TC
                         ? net_limb_layer(net, L, cur)
                         : rss_matmul<uint64_t>(c, cur, (const uint64_t *const *)L.w, L.out, bias, net->batch, L.p[1],
                                                L.p[0], 1, 1, 1, net->fp);
                break;
            }
            case PG_LAYER_CNN:
                st = c->form == PG_FORM_LIMB_TC
                         ? net_limb_layer(net, L, cur)
                         : rss_conv<uint64_t>(c, cur, (const uint64_t *const *)L.w, L.out, PG_CONV_FPROP, net->batch,
                                              L.p[0], L.p[1], L.p[4], L.p[2], L.p[3], L.p[5], L.p[6], net->fp);
                break;
            case PG_LAYER_RELU: st = rss_relu<uint64_t, uint8_t>(c, cur, L.in_n, L.out, L.d); break;
            case PG_LAYER_MAXPOOL:
                st = rss_maxpool_layer<uint64_t, uint8_t>(c, cur, L.out, L.d, L.p[0], L.p[1], L.p[2], L.p[3], L.p[4],
                                                          net->batch, net->fp);
                break;
            default: st = set_error(c, PG_ERR_INVALID_ARG, "bad layer type %d", L.type);
        }
        if (st) return st;
        if (!net->ev.empty() && (st = record_event(c, net->ev[2 * li + 1]))) return st;
        cur = L.out;
    }
    return PG_OK;
}

extern "C" {

int pg_net_create(pg_ctx *c, pg_net **out, const int *spec, int nlayers, int batch, int fp) {
    if (!c || !out || !spec || nlayers <= 0 || batch <= 0 || fp < 0 || fp > 62) return PG_ERR_INVALID_ARG;
    *out = nullptr;
    pg_net *net = new pg_net();
    net->ctx = c;
    net->batch = batch;
    net->fp = fp;
    size_t cur_n = 0;  // elements per share of the running activation
    for (int i = 0; i < nlayers; i++) {
        NetLayer L;
        memset(&L, 0, sizeof(L));
        L.type = spec[8 * i];
        for (int k = 0; k < 7; k++) L.p[k] = spec[8 * i + 1 + k];
        switch (L.type) {
            case PG_LAYER_FC:
                L.in_n = (size_t)batch * L.p[0];
                L.out_n = (size_t)batch * L.p[1];
                L.w_n = (size_t)L.p[0] * L.p[1];
                L.b_n = L.p[1];
                break;
            case PG_LAYER_CNN: {
                int H = L.p[0], W = L.p[1], Din = L.p[2], Dout = L.p[3], f = L.p[4], s = L.p[5], pd = L.p[6];
                if (H <= 0 || W <= 0 || Din <= 0 || Dout <= 0 || f <= 0 || s <= 0 || pd < 0 || H + 2 * pd < f ||
                    W + 2 * pd < f) {
                    delete net;
                    return set_error(c, PG_ERR_SIZE, "layer %d: bad conv geometry", i);
                }
                int P = (H + 2 * pd - f) / s + 1, Q = (W + 2 * pd - f) / s + 1;
                L.in_n = (size_t)batch * H * W * Din;
                L.out_n = (size_t)batch * P * Q * Dout;
                L.w_n = (size_t)Dout * f * f * Din;
                break;
            }
            case PG_LAYER_RELU:
                L.in_n = L.out_n = (size_t)batch * L.p[0];
                L.d_n = L.out_n;
                break;
            case PG_LAYER_MAXPOOL: {
                int H = L.p[0], W = L.p[1], C = L.p[2], f = L.p[3], s = L.p[4];
                if (f <= 0 || s <= 0 || f > H || f > W) {
                    delete net;
                    return set_error(c, PG_ERR_SIZE, "layer %d: bad pool geometry", i);
                }
                L.in_n = (size_t)batch * H * W * C;
                L.out_n = (size_t)batch * ((H - f) / s + 1) * ((W - f) / s + 1) * C;
                L.d_n = L.out_n * f * f;
                break;
            }
            default: delete net; return set_error(c, PG_ERR_INVALID_ARG, "layer %d: bad type %d", i, L.type);
        }
        if (i > 0 && L.in_n != cur_n) {
            delete net;
            return set_error(c, PG_ERR_SIZE, "layer %d expects %zu inputs per share, previous layer gives %zu", i, L.in_n,
                             cur_n);
        }
        if (i == 0) net->in_n = L.in_n;
        cur_n = L.out_n;
        net->layers.push_back(L);
    }
    net->out_n = cur_n;
    // one arena: input, then per layer weights, bias, outputs, bits (256-byte aligned pieces)
    auto al = [](size_t b) { return (b + 255) & ~(size_t)255; };
    size_t bytes = 6 * al(net->in_n * 8);
    for (auto &L : net->layers) bytes += 6 * (al(L.w_n * 8) + al(L.b_n * 8) + al(L.out_n * 8) + al(L.d_n));
    if (cudaMalloc(&net->arena, bytes) != cudaSuccess) {
        cudaGetLastError();
        delete net;
        return set_error(c, PG_ERR_NO_MEMORY, "network arena of %zu bytes", bytes);
    }
    net->arena_bytes = bytes;
    cudaMemsetAsync(net->arena, 0, bytes, c->stream);
    char *ptr = (char *)net->arena;
    // input shares contiguous [6][in_n] so host copies are one transfer
    for (int k = 0; k < 6; k++) net->in[k] = (uint64_t *)(ptr + k * net->in_n * 8);
    ptr += al(6 * net->in_n * 8);
    for (auto &L : net->layers) {
        for (int k = 0; k < 6; k++) { L.w[k] = (uint64_t *)ptr; ptr += al(L.w_n * 8); }
        for (int k = 0; k < 6; k++) { L.b[k] = L.b_n ? (uint64_t *)ptr : nullptr; ptr += al(L.b_n * 8); }
        char *o = ptr;
        for (int k = 0; k < 6; k++) L.out[k] = (uint64_t *)(o + k * L.out_n * 8);
        ptr += al(6 * L.out_n * 8);
        for (int k = 0; k < 6; k++) { L.d[k] = L.d_n ? (uint8_t *)ptr : nullptr; ptr += al(L.d_n); }
    }
    *out = net;
    return PG_OK;
}

int pg_net_destroy(pg_net *net) {
    if (!net) return PG_ERR_INVALID_ARG;
    for (auto e : net->ev) cudaEventDestroy(e);
    if (net->exec) cudaGraphExecDestroy(net->exec);
    if (net->graph) cudaGraphDestroy(net->graph);
    if (net->arena || net->limb_arena) cudaStreamSynchronize(net->ctx->stream);
    if (net->arena) cudaFree(net->arena);
    if (net->limb_arena) cudaFree(net->limb_arena);
    delete net;
    return PG_OK;
}

int pg_net_set_params(pg_net *net, int layer, const uint64_t *const w[6], const uint64_t *const bias[6]) {
    if (!net || layer < 0 || layer >= (int)net->layers.size()) return PG_ERR_INVALID_ARG;
    NetLayer &L = net->layers[layer];
    Ctx *c = net->ctx;
    if (L.w_n) {
        if (!w) return set_error(c, PG_ERR_INVALID_ARG, "layer %d needs weights", layer);
        for (int k = 0; k < 6; k++)
            PG_CHECK_CUDA(c, cudaMemcpyAsync(L.w[k], w[k], L.w_n * 8, cudaMemcpyDeviceToDevice, c->stream));
    }
    if (L.b_n && bias)
        for (int k = 0; k < 6; k++)
            PG_CHECK_CUDA(c, cudaMemcpyAsync(L.b[k], bias[k], L.b_n * 8, cudaMemcpyDeviceToDevice, c->stream));
    // the limb form keeps the weights packed: repack this layer's
    if (net->limb_arena && L.packB) {
        int st = lt::run_pack(c, L.plan, (const uint64_t *const *)L.w, L.packB);
        if (st) return st;
    }
    // a set-up call: the caller may release the source buffers on return
    PG_CHECK_CUDA(c, cudaStreamSynchronize(c->stream));
    return PG_OK;
}

size_t pg_net_input_size(pg_net *net) { return net ? net->in_n : 0; }
size_t pg_net_output_size(pg_net *net) { return net ? net->out_n : 0; }

int pg_net_forward(pg_net *net, const uint64_t *const in[6], uint64_t *const out[6]) {
    if (!net || !in || !out) return PG_ERR_INVALID_ARG;
    Ctx *c = net->ctx;
    int st = net_run(net, in);
    if (st) return st;
    NetLayer &last = net->layers.back();
    for (int k = 0; k < 6; k++)
        if (out[k] != last.out[k])
            PG_CHECK_CUDA(c, cudaMemcpyAsync(out[k], last.out[k], net->out_n * 8, cudaMemcpyDeviceToDevice, c->stream));
    return PG_OK;
}

int pg_net_capture(pg_net *net) {
    if (!net) return PG_ERR_INVALID_ARG;
    Ctx *c = net->ctx;
    if (net->exec) {
        cudaGraphExecDestroy(net->exec);
        net->exec = nullptr;
    }
    if (net->graph) {
        cudaGraphDestroy(net->graph);
        net->graph = nullptr;
    }
    // One eager forward first: it sizes the context scratch (split-K
    // partials), which cannot be allocated while a stream is capturing.
    {
        uint64_t comm_save[9];
        memcpy(comm_save, c->comm, sizeof(comm_save));
        uint64_t launches_save = c->launches.load();
        int st0 = net_run(net, (const uint64_t *const *)net->in);
        memcpy(c->comm, comm_save, sizeof(comm_save));
        c->launches = launches_save;
        if (st0) return st0;
        PG_CHECK_CUDA(c, cudaStreamSynchronize(c->stream));
    }
    // Capture on a private stream (the context stream may be the legacy
    // default stream, which cannot be captured); replays go to ctx->stream.
    cudaStream_t cap = nullptr, user = c->stream;
    PG_CHECK_CUDA(c, cudaStreamCreateWithFlags(&cap, cudaStreamNonBlocking));
    cudaEvent_t ev = nullptr;
    PG_CHECK_CUDA(c, cudaEventCreateWithFlags(&ev, cudaEventDisableTiming));
    cudaEventRecord(ev, user);
    cudaStreamWaitEvent(cap, ev, 0);
    uint64_t comm_before[9];
    memcpy(comm_before, c->comm, sizeof(comm_before));
    uint64_t launches_before = c->launches.load();
    c->stream = cap;
    cudaError_t e0 = cudaStreamBeginCapture(cap, cudaStreamCaptureModeThreadLocal);
    int st = e0 == cudaSuccess ? net_run(net, (const uint64_t *const *)net->in) : PG_ERR_CUDA;
    cudaGraph_t g = nullptr;
    cudaError_t e = e0 == cudaSuccess ? cudaStreamEndCapture(cap, &g) : e0;
    c->stream = user;
    cudaStreamSynchronize(cap);
    cudaStreamDestroy(cap);
    cudaEventDestroy(ev);
    for (int k = 0; k < 9; k++) net->comm_per_fwd[k] = c->comm[k] - comm_before[k];
    memcpy(c->comm, comm_before, sizeof(comm_before));
    uint64_t launched = c->launches.load() - launches_before;
    c->launches = launches_before;
    if (st) {
        if (g) cudaGraphDestroy(g);
        return st;
    }
    if (e != cudaSuccess) return set_error(c, PG_ERR_CUDA, "graph capture: %s", cudaGetErrorString(e));
    net->graph = g;
    PG_CHECK_CUDA(c, cudaGraphInstantiate(&net->exec, g, 0));
    net->launches_per_fwd = launched;  // capture does not execute: replays add these
    return PG_OK;
}

static int net_replay_or_run(pg_net *net) {
    Ctx *c = net->ctx;
    if (net->exec) {
        PG_CHECK_CUDA(c, cudaGraphLaunch(net->exec, c->stream));
        for (int k = 0; k < 9; k++) c->comm[k] += net->comm_per_fwd[k];
        c->launches += net->launches_per_fwd;
        return PG_OK;
    }
    return net_run(net, (const uint64_t *const *)net->in);
}

int pg_net_forward_host(pg_net *net, const uint64_t *in_host, uint64_t *out_host) {
    if (!net || !in_host || !out_host) return PG_ERR_INVALID_ARG;
    Ctx *c = net->ctx;
    PG_CHECK_CUDA(c, cudaMemcpyAsync(net->in[0], in_host, 6 * net->in_n * 8, cudaMemcpyHostToDevice, c->stream));
    int st = net_replay_or_run(net);
    if (st) return st;
    NetLayer &last = net->layers.back();
    PG_CHECK_CUDA(c, cudaMemcpyAsync(out_host, last.out[0], 6 * net->out_n * 8, cudaMemcpyDeviceToHost, c->stream));
    return PG_OK;
}

int pg_net_forward_resident(pg_net *net) {
    if (!net) return PG_ERR_INVALID_ARG;
    return net_replay_or_run(net);
}

int pg_net_input_shares(pg_net *net, uint64_t *out[6]) {
    if (!net || !out) return PG_ERR_INVALID_ARG;
    for (int k = 0; k < 6; k++) out[k] = net->in[k];
    return PG_OK;
}

int pg_net_enable_timing(pg_net *net, int on) {
    if (!net) return PG_ERR_INVALID_ARG;
    if (net->exec) return set_error(net->ctx, PG_ERR_INVALID_ARG, "enable timing before capturing the graph");
    for (auto e : net->ev) cudaEventDestroy(e);
    net->ev.clear();
    if (on) {
        net->ev.resize(2 * net->layers.size());
        for (auto &e : net->ev) PG_CHECK_CUDA(net->ctx, cudaEventCreate(&e));
    }
    return PG_OK;
}

int pg_net_layer_times(pg_net *net, float *ms) {
    if (!net || !ms) return PG_ERR_INVALID_ARG;
    if (net->ev.empty()) return set_error(net->ctx, PG_ERR_INVALID_ARG, "per-layer timing is off");
    for (size_t i = 0; i < net->layers.size(); i++)
        PG_CHECK_CUDA(net->ctx, cudaEventElapsedTime(&ms[i], net->ev[2 * i], net->ev[2 * i + 1]));
    return PG_OK;
}

int pg_net_layer_output(pg_net *net, int layer, uint64_t *const out[6], size_t *n) {
    if (!net || layer < 0 || layer >= (int)net->layers.size()) return PG_ERR_INVALID_ARG;
    NetLayer &L = net->layers[layer];
    if (out)
        for (int k = 0; k < 6; k++) ((uint64_t **)out)[k] = L.out[k];
    if (n) *n = L.out_n;
    return PG_OK;
}

}  // extern "C"
