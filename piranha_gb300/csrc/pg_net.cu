// pg_net.cu — network executor: NeuralNetwork::forward (src/nn/NeuralNetwork.cu:109-133)
// and ::backward (:136-148, :207-267, :439-460) over FC / CNN / ReLU / Maxpool
// layers (FCLayer.cu:78-217, CNNLayer.cu:81-193, ReLULayer.cu:51-124,
// MaxpoolLayer.cu:52-185). All share buffers of all layers are allocated once
// in one device arena at creation (the training buffers in a second one, on
// first use); a forward or a training step is a fixed sequence of fused
// launches on the context stream, which pg_net_capture / pg_net_capture_train
// record as one CUDA graph so that a replay costs one launch.
#include <cmath>
#include <cstring>
#include <limits>
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
template <typename T, typename U>
int rss_select(Ctx *, const T *const *, const T *const *, const U *const *, T *const *, size_t);
template <typename T>
int rss_avgpool_layer(Ctx *, const T *const *, T *const *, int, int, int, int, int, int);
template <typename T>
int rss_avgpool_backward(Ctx *, const T *const *, T *const *, int, int, int, int, int, int);
template <typename T> int rss_reconstruct(Ctx *, const T *const *, size_t, T *const *);
template <typename T> int rss_divide_public(Ctx *, T *const *, size_t, T, const T *);
int reduce_sum_u64(Ctx *, const uint64_t *, uint64_t *, int, int, int);
int limb3_rss_matmul_u64(Ctx *, const uint64_t *const *, const uint64_t *const *, uint64_t *const *,
                         const uint64_t *const *, int, int, int, int, int, int, int);
int limb3_rss_conv_u64(Ctx *, const uint64_t *const *, const uint64_t *const *, uint64_t *const *, int, int, int, int,
                       int, int, int, int, int, int);
void count_relu_u64_u8(Ctx *, size_t);
}  // namespace pg

using namespace pg;

struct NetLayer {
    int type;
    int p[7];
    size_t in_n, out_n, w_n, b_n, d_n;  // elements per share buffer (activations include the batch)
    uint64_t *w[6], *b[6], *out[6];
    uint8_t *d[6];
    uint64_t *delta[6];  // backward: the gradient this layer passes to the previous one (in_n)
    // limb tensor-core form (FC and CNN layers): plan, split-K, packed weights
    lt::Plan plan;
    lt::Plan alt;      // a position-major convolution's rectangle-tile plan, timed against it at set-up
    bool has_alt = false;
    int split, cps;
    uint8_t *packB;
    int u64 = 0;  // the plain u64 form timed faster for this layer at set-up (small layers)
    bool b_replicated = true;  // the bias shares are a replicated sharing (checked by pg_net_set_params)
    bool out_rep = false;      // the last forward left a replicated sharing in out (see net_run)
    // A CNN layer after a ReLU: its own digit image, which that ReLU writes
    // (relu_image) and which keeps the ReLU's output between forwards;
    // held_shared: the image's three-block layout (a replicated sharing).
    uint8_t *held = nullptr;
    bool held_shared = false;
    // A ReLU layer that writes the next layer's held image: an inference
    // forward keeps its output there alone (out[] is rebuilt from the image
    // when it is read); a training forward writes out[] too
    bool out_held = false;
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
    // pg_net_forward_host with a captured forward: a second input buffer set
    // and its own captured graph, so that the next call's host-to-device copy
    // (on the copy stream) overlaps the current replay
    uint64_t *in_alt = nullptr;
    cudaGraph_t graph_alt = nullptr;
    cudaGraphExec_t exec_alt = nullptr;
    cudaStream_t copy = nullptr;
    cudaEvent_t in_ready[2] = {nullptr, nullptr}, in_free[2] = {nullptr, nullptr};
    int slot = 0;
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
    // The last forward that ran (eager or a replay) was an inference forward
    // (no training buffers): the ReLU / maxpool bit shares were not written,
    // nor the out[] of the ReLUs marked out_held. fwd_graph_held: the same
    // for the captured forward graphs.
    bool last_fwd_held = false, fwd_graph_held = false;
    int *in_rep = nullptr;  // device word: the forward's input is a replicated sharing (checked each forward)
    uint64_t *limb_partial = nullptr;
    // Training (allocated by the first training call, which is eager):
    struct Train {
        void *arena = nullptr;
        uint64_t *labels[6];   // label shares [6][out_n], contiguous
        uint64_t *sdelta[6];   // the softmax gradient [6][out_n]
        uint64_t *rev[3];      // each party's reveal of the logits
        uint64_t *sm[3];       // each party's softmax, fixed point
        uint64_t *h_rev = nullptr, *h_sm = nullptr;  // pinned host copies [3][out_n]
        uint64_t *dW[6], *db[6];  // FC / CNN parameter gradients
        uint64_t *pools[6];       // maxpool: incoming gradient expanded over each window
        uint64_t *zeros;          // shared zero operand of selectShare
        uint64_t *backup;         // parameter snapshot around the capture's eager run
        size_t backup_bytes = 0;
        // host softmax job (stable address: a graph host node points at it)
        size_t n = 0;
        int batch = 0, fp = 0;
    } tr;
    cudaGraph_t graph_train = nullptr;
    cudaGraphExec_t exec_train = nullptr;
    uint64_t comm_per_train[9] = {0};
    uint64_t launches_per_train = 0;
};

// The tile shape of a convolution that position-major tiles apply to: the
// position-major plan (one output pixel of 128 images per tile, only the
// taps inside the input) and the rectangle plan (128 pixels of one or more
// images per tile, every tap), each with its own tuned split-K, timed on the
// zero image into the layer's outputs (one warm-up, three timed runs each);
// the rectangle plan is kept only if it wins by 3 %. The choice is cached
// with the split-K choices (1 = rectangle, 2 = position-major). The next
// layer's fused ReLU writes the image in the chosen plan's layout. Without
// autotuning the position-major plan stays.
static int net_choose_tiles(pg_net *net, NetLayer &L, const uint64_t *const *bias) {
    Ctx *c = net->ctx;
    const std::string key = "tile/" + lt::plan_key(L.alt);
    int choice = 2;
    auto it = c->split_cache.find(key);
    if (it != c->split_cache.end()) {
        choice = it->second.first;
    } else if (c->autotune) {
        int split[2] = {L.split, 0}, cps[2] = {L.cps, 0};
        int st = lt::tune_split(c, L.alt, net->limb_image, L.packB, net->limb_partial, L.out, bias, net->fp,
                                bias == nullptr, nullptr, split[1], cps[1]);
        if (st) return st;
        cudaEvent_t e0, e1;
        PG_CHECK_CUDA(c, cudaEventCreate(&e0));
        if (cudaEventCreate(&e1) != cudaSuccess) {
            cudaEventDestroy(e0);
            return set_error(c, PG_ERR_CUDA, "cudaEventCreate failed");
        }
        float ms[2] = {0.f, 0.f};
        for (int v = 0; v < 2 && !st; v++) {
            const lt::Plan &p = v ? L.alt : L.plan;
            for (int r = 0; r < 4 && !st; r++) {
                if (r == 1 && cudaEventRecord(e0, c->stream) != cudaSuccess) st = set_error(c, PG_ERR_CUDA, "event");
                if (!st)
                    st = lt::run_gemm(c, p, net->limb_image, L.packB, split[v] > 1 ? net->limb_partial : nullptr,
                                      split[v], cps[v], L.out, bias, net->fp, bias == nullptr);
            }
            if (!st && cudaEventRecord(e1, c->stream) != cudaSuccess) st = set_error(c, PG_ERR_CUDA, "event");
            if (!st && cudaEventSynchronize(e1) != cudaSuccess) st = set_error(c, PG_ERR_CUDA, "event");
            if (!st && cudaEventElapsedTime(&ms[v], e0, e1) != cudaSuccess) st = set_error(c, PG_ERR_CUDA, "event");
        }
        cudaEventDestroy(e0);
        cudaEventDestroy(e1);
        if (st) return st;
        choice = ms[1] < 0.97f * ms[0] ? 1 : 2;
        c->split_cache[key] = {choice, 1};
    }
    if (choice == 1) {
        L.plan = L.alt;
        int sp, cp;
        if (lt::cached_split(c, L.plan, sp, cp)) {
            L.split = sp;
            L.cps = cp;
        } else {
            lt::choose_split(L.plan, c->sm_count > 0 ? c->sm_count : 148, L.split, L.cps);
        }
    }
    L.has_alt = false;
    return PG_OK;
}

// The digit image a CNN layer owns when the ReLU before it can write it
// (either tile plan: the set-up timing picks one of them afterwards).
static size_t held_bytes(pg_net *net, NetLayer &L) {
    if (L.type != PG_LAYER_CNN) return 0;
    const size_t li = (size_t)(&L - net->layers.data());
    if (li == 0 || net->layers[li - 1].type != PG_LAYER_RELU) return 0;
    const size_t n = net->layers[li - 1].in_n;
    size_t b = lt::relu_image_fits(L.plan, n) ? L.plan.image_bytes : 0;
    if (L.has_alt && lt::relu_image_fits(L.alt, n) && L.alt.image_bytes > b) b = L.alt.image_bytes;
    return b;
}

// Plans, buffer sizes and weight packing of the limb form.
static int net_limb_setup(pg_net *net) {
    Ctx *c = net->ctx;
    auto al = [](size_t b) { return (b + 255) & ~(size_t)255; };
    size_t image = 0, partial = 0, packs = 0, held = 0;
    const int sms = c->sm_count > 0 ? c->sm_count : 148;
    for (auto &L : net->layers) {
        int st = PG_OK;
        if (L.type == PG_LAYER_FC) st = lt::plan_gemm(c, L.plan, net->batch, L.p[1], L.p[0], 1, 1, 1);
        else if (L.type == PG_LAYER_CNN) {
            st = lt::plan_conv(c, L.plan, net->batch, L.p[0], L.p[1], L.p[4], L.p[2], L.p[3], L.p[5], L.p[6]);
            L.has_alt = false;
            if (!st && L.plan.posmajor) {
                st = lt::plan_conv(c, L.alt, net->batch, L.p[0], L.p[1], L.p[4], L.p[2], L.p[3], L.p[5], L.p[6],
                                   false);
                L.has_alt = st == PG_OK;
            }
        } else continue;
        if (st) return st;
        lt::choose_split(L.plan, sms, L.split, L.cps);
        image = image > L.plan.image_bytes ? image : L.plan.image_bytes;
        held += al(held_bytes(net, L));
        size_t pb = lt::tune_partial_bytes(L.plan, sms);
        if (L.has_alt) {
            // the same packed weights and image size; its own split-K candidates
            image = image > L.alt.image_bytes ? image : L.alt.image_bytes;
            const size_t pa = lt::tune_partial_bytes(L.alt, sms);
            pb = pb > pa ? pb : pa;
        }
        partial = partial > pb ? partial : pb;
        packs += al(L.plan.packB_bytes);
    }
    const size_t bytes = al(image) + al(partial) + packs + held + 256;
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
    net->in_rep = (int *)ptr;
    ptr += 256;
    for (auto &L : net->layers) {
        if (L.type != PG_LAYER_FC && L.type != PG_LAYER_CNN) continue;
        L.packB = ptr;
        ptr += al(L.plan.packB_bytes);
        int st = lt::run_pack(c, L.plan, (const uint64_t *const *)L.w, L.packB);
        if (st) return st;
    }
    for (auto &L : net->layers) {
        const size_t hb = held_bytes(net, L);
        if (!hb) continue;
        L.held = ptr;
        ptr += al(hb);
        // rows past the activation stay 0 (the GEMM's last tile line reads them)
        PG_CHECK_CUDA(c, cudaMemsetAsync(L.held, 0, al(hb), c->stream));
    }
    // split-K of every layer, timed on a zero image into the layer's own
    // outputs (the forward overwrites them; without a bias only the value
    // shares are written, so the zero shares stay 0)
    PG_CHECK_CUDA(c, cudaMemsetAsync(net->limb_image, 0, al(image), c->stream));
    for (auto &L : net->layers) {
        if (L.type != PG_LAYER_FC && L.type != PG_LAYER_CNN) continue;
        const uint64_t *const *bias = L.b_n ? (const uint64_t *const *)L.b : nullptr;
        int st = lt::tune_split(c, L.plan, net->limb_image, L.packB, net->limb_partial, L.out, bias, net->fp,
                                bias == nullptr, nullptr, L.split, L.cps);
        if (st) return st;
        if (L.has_alt && (st = net_choose_tiles(net, L, bias))) return st;
    }
    return PG_OK;
}

// One FC / CNN layer in the limb form: digit image of the input, GEMM over
// the packed weights (+ split-K reduction), then the message accounting of
// matmul / convolution (RSS.inl:517-538, :790-802).
// shared: the input's six buffers hold a replicated sharing (every layer
// output of the network does: an FC / CNN output is [v, 0, 0, 0, 0, v], and
// the ReLU, maxpool and averagepool steps keep a replicated sharing
// replicated), so the digit image stores each of the three shares once.
// rep_flag: a device word that says whether in[] holds a replicated sharing
// (the network's input, checked on the device each forward)
static int net_limb_layer(pg_net *net, NetLayer &L, const uint64_t *const *in, bool image_ready = false,
                          bool shared = false, const int *rep_flag = nullptr) {
    Ctx *c = net->ctx;
    // the ReLU before it wrote the image into the layer's own buffer
    uint8_t *const image = image_ready && L.held ? L.held : net->limb_image;
    int st = image_ready ? PG_OK : lt::run_image(c, L.plan, in, image, shared, rep_flag);
    if (st) return st;
    const uint64_t *const *bias = L.b_n ? (const uint64_t *const *)L.b : nullptr;
    // The arena is zeroed when the network is created and a layer's output
    // buffers are written by that layer alone, so without a bias the four
    // shares that dividePublic3out3 leaves at 0 stay 0: write only the two
    // value shares.
    st = lt::run_gemm(c, L.plan, image, L.packB, L.split > 1 ? net->limb_partial : nullptr, L.split, L.cps,
                      L.out, bias, net->fp, bias == nullptr, nullptr, shared, image_ready ? nullptr : rep_flag);
    if (st) return st;
    const uint64_t n_out = (uint64_t)L.plan.M * L.plan.N;
    comm_msg(c, 2 * n_out * 8, 2 * n_out * 8);
    comm_round(c);
    return PG_OK;
}

// The same FC / CNN layer in the plain u64 form (FCLayer.cu:101-116,
// CNNLayer.cu:95-99).
static int net_u64_layer(pg_net *net, NetLayer &L, const uint64_t *const *in) {
    Ctx *c = net->ctx;
    if (L.type == PG_LAYER_FC) {
        const uint64_t *const *bias = L.b_n ? (const uint64_t *const *)L.b : nullptr;
        return rss_matmul<uint64_t>(c, in, (const uint64_t *const *)L.w, L.out, bias, net->batch, L.p[1], L.p[0], 1,
                                    1, 1, net->fp);
    }
    return rss_conv<uint64_t>(c, in, (const uint64_t *const *)L.w, L.out, PG_CONV_FPROP, net->batch, L.p[0], L.p[1],
                              L.p[4], L.p[2], L.p[3], L.p[5], L.p[6], net->fp);
}

// Per FC / CNN layer of a limb-form network, the form that runs it faster:
// both are timed on the layer's own buffers (one warm-up, then three runs
// each, CUDA events on the context's stream; the outputs are overwritten by
// the first real forward), and the u64 form is kept only if it wins by 3 %.
// Both compute the same bits. Communication and launch counters are restored.
static int net_choose_forms(pg_net *net) {
    Ctx *c = net->ctx;
    if (!c->autotune) return PG_OK;
    uint64_t comm0[9];
    memcpy(comm0, c->comm, sizeof(comm0));
    const uint64_t launches0 = c->launches.load();
    cudaEvent_t e0, e1;
    PG_CHECK_CUDA(c, cudaEventCreate(&e0));
    if (cudaEventCreate(&e1) != cudaSuccess) {
        cudaEventDestroy(e0);
        return set_error(c, PG_ERR_CUDA, "cudaEventCreate failed");
    }
    int st = PG_OK;
    for (size_t li = 0; li < net->layers.size() && !st; li++) {
        NetLayer &L = net->layers[li];
        if (L.type != PG_LAYER_FC && L.type != PG_LAYER_CNN) continue;
        // the choice is cached with the split-K choices (and so in a tuning
        // cache file): 1 = limb form, 2 = u64 form
        const std::string key = "form/" + std::to_string(L.type) + "/" + lt::plan_key(L.plan);
        auto it = c->split_cache.find(key);
        if (it != c->split_cache.end()) {
            L.u64 = it->second.first == 2;
            continue;
        }
        const uint64_t *const *in = li ? (const uint64_t *const *)net->layers[li - 1].out
                                       : (const uint64_t *const *)net->in;
        float ms[2] = {0.f, 0.f};
        for (int form = 0; form < 2 && !st; form++) {
            for (int r = 0; r < 4 && !st; r++) {
                if (r == 1 && cudaEventRecord(e0, c->stream) != cudaSuccess) st = set_error(c, PG_ERR_CUDA, "event");
                if (!st) st = form ? net_u64_layer(net, L, in) : net_limb_layer(net, L, in);
            }
            if (!st && cudaEventRecord(e1, c->stream) != cudaSuccess) st = set_error(c, PG_ERR_CUDA, "event");
            if (!st && cudaEventSynchronize(e1) != cudaSuccess) st = set_error(c, PG_ERR_CUDA, "event");
            if (!st && cudaEventElapsedTime(&ms[form], e0, e1) != cudaSuccess) st = set_error(c, PG_ERR_CUDA, "event");
        }
        if (!st) {
            L.u64 = ms[1] < 0.97f * ms[0];
            c->split_cache[key] = {L.u64 ? 2 : 1, 1};
        }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    // the zero shares of a limb layer's output stay 0 only if the u64 runs did
    // not leave values there: the u64 form writes every share, with the same
    // zeros, so they are still 0
    memcpy(c->comm, comm0, sizeof(comm0));
    c->launches.store(launches0);
    return st;
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

static int check_replicated(Ctx *c, const uint64_t *const in[6], size_t n, int *flag);

static int net_run(pg_net *net, const uint64_t *const in[6]) {
    Ctx *c = net->ctx;
    const uint64_t *const *cur = in;
    if (c->form == PG_FORM_LIMB_TC && !net->limb_arena) {
        cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
        PG_CHECK_CUDA(c, cudaStreamIsCapturing(c->stream, &cs));
        if (cs != cudaStreamCaptureStatusNone)
            return set_error(c, PG_ERR_INVALID_ARG, "limb-form buffers must be set up by an eager forward first");
        int st = net_limb_setup(net);
        if (!st) st = net_choose_forms(net);
        if (st) return st;
    }
    // Whether the caller's input is a replicated sharing is checked on the
    // device (one read of the six buffers) where the first layer's digit image
    // can use it: its image kernel and GEMM read the answer.
    const int *in_rep = nullptr;
    if (c->form == PG_FORM_LIMB_TC && net->in_rep && !net->layers.empty() &&
        (net->layers[0].type == PG_LAYER_FC || net->layers[0].type == PG_LAYER_CNN) && !net->layers[0].u64) {
        int st = check_replicated(c, in, net->in_n, net->in_rep);
        if (st) return st;
        in_rep = net->in_rep;
    }
    // An inference forward (no training buffers, so no backward follows it)
    // writes no bit shares, and a ReLU that writes the next convolution's
    // digit image keeps its output there alone.
    const bool hold = !net->tr.arena;
    bool ready_next = false;  // the previous ReLU wrote this layer's digit image
    bool zero_mid = false;    // cur's shares 1-4 are 0 (the previous layer is a bias-free FC / CNN)
    // The network's input is taken as six independent buffers; an FC / CNN
    // output is a replicated sharing ([v, 0, 0, 0, 0, v] plus the bias shares,
    // when those are replicated too), and the layers after it keep it so.
    bool replicated = false;
    for (size_t li = 0; li < net->layers.size(); li++) {
        NetLayer &L = net->layers[li];
        int st = PG_OK;
        const bool image_ready = ready_next;
        ready_next = false;
        L.out_held = false;
        if (!net->ev.empty() && (st = record_event(c, net->ev[2 * li]))) return st;
        switch (L.type) {
            case PG_LAYER_FC: {
                const uint64_t *const *bias = L.b_n ? (const uint64_t *const *)L.b : nullptr;
                st = c->form == PG_FORM_LIMB_TC
                         ? (L.u64 ? net_u64_layer(net, L, cur)
                                  : net_limb_layer(net, L, cur, false, replicated, li == 0 ? in_rep : nullptr))
                         : rss_matmul<uint64_t>(c, cur, (const uint64_t *const *)L.w, L.out, bias, net->batch, L.p[1],
                                                L.p[0], 1, 1, 1, net->fp);
                break;
            }
            case PG_LAYER_CNN:
                st = c->form == PG_FORM_LIMB_TC
                         ? (L.u64 ? net_u64_layer(net, L, cur)
                                  : net_limb_layer(net, L, cur, image_ready, replicated, li == 0 ? in_rep : nullptr))
                         : rss_conv<uint64_t>(c, cur, (const uint64_t *const *)L.w, L.out, PG_CONV_FPROP, net->batch,
                                              L.p[0], L.p[1], L.p[4], L.p[2], L.p[3], L.p[5], L.p[6], net->fp);
                break;
            case PG_LAYER_RELU: {
                // a ReLU that feeds a limb-form implicit convolution also writes
                // that convolution's digit image (the layer outputs as before)
                NetLayer *next = li + 1 < net->layers.size() ? &net->layers[li + 1] : nullptr;
                if (c->form == PG_FORM_LIMB_TC && net->limb_arena && next && next->type == PG_LAYER_CNN &&
                    !next->u64 && lt::relu_image_fits(next->plan, L.in_n)) {
                    uint8_t *const image = next->held ? next->held : net->limb_image;
                    L.out_held = next->held != nullptr;
                    c->in_zero_mid = zero_mid;
                    st = lt::run_relu_image(c, next->plan, cur, L.in_n, hold && L.out_held ? nullptr : L.out,
                                            hold ? nullptr : L.d, image, replicated);
                    c->in_zero_mid = false;
                    if (!st) count_relu_u64_u8(c, L.in_n);
                    ready_next = !st;
                    next->held_shared = replicated;
                } else {
                    st = rss_relu<uint64_t, uint8_t>(c, cur, L.in_n, L.out, hold ? nullptr : L.d);
                }
                break;
            }
            case PG_LAYER_MAXPOOL:
                c->in_zero_mid = zero_mid;
                st = rss_maxpool_layer<uint64_t, uint8_t>(c, cur, L.out, hold ? nullptr : L.d, L.p[0], L.p[1], L.p[2],
                                                          L.p[3], L.p[4], net->batch, net->fp);
                c->in_zero_mid = false;
                break;
            case PG_LAYER_AVGPOOL:
                st = rss_avgpool_layer<uint64_t>(c, cur, L.out, L.p[0], L.p[1], L.p[2], L.p[3], L.p[4], net->batch);
                break;
            default: st = set_error(c, PG_ERR_INVALID_ARG, "bad layer type %d", L.type);
        }
        if (st) return st;
        if (!net->ev.empty() && (st = record_event(c, net->ev[2 * li + 1]))) return st;
        if (L.type == PG_LAYER_FC || L.type == PG_LAYER_CNN) replicated = !L.b_n || L.b_replicated;
        L.out_rep = replicated;
        // dividePublic3out3 leaves party A's shareB, party B's shares and party
        // C's shareA at 0 (and the network never writes them), unless a bias
        // share is added there
        zero_mid = (L.type == PG_LAYER_FC || L.type == PG_LAYER_CNN) && !L.b_n;
        cur = L.out;
    }
    net->last_fwd_held = hold;
    return PG_OK;
}

// ------------------------------------------------------------- training

namespace {

__global__ void softmax_delta_kernel(Sh6<uint64_t> out, const uint64_t *smA, const uint64_t *smC, CSh6<uint64_t> lab,
                                     size_t n) {
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
        // deltas = 0; deltas += softmax (party A shareA, party C shareB); deltas -= labels
        out.p[0][i] = smA[i] - lab.p[0][i];
        out.p[1][i] = 0 - lab.p[1][i];
        out.p[2][i] = 0 - lab.p[2][i];
        out.p[3][i] = 0 - lab.p[3][i];
        out.p[4][i] = 0 - lab.p[4][i];
        out.p[5][i] = smC[i] - lab.p[5][i];
    }
}

// FCLayer::backward's bias gradient (FCLayer.cu:184-189: db zeroed, then
// reduceSum(delta, db, false, outputDim, batchSize)) of all six shares in one
// launch: db[k][c] = sum over i < len of delta[k][c * len + i], block (k, c)
// per output.
__global__ void bias_grad6_kernel(CSh6<uint64_t> d, Sh6<uint64_t> db, int outn, int len) {
    __shared__ uint64_t red[256];
    for (int blk = blockIdx.x; blk < 6 * outn; blk += gridDim.x) {
        const int k = blk / outn, col = blk - k * outn;
        uint64_t acc = 0;
        for (int i = threadIdx.x; i < len; i += blockDim.x) acc += d.p[k][(size_t)len * col + i];
        red[threadIdx.x] = acc;
        __syncthreads();
        for (int s = blockDim.x / 2; s > 0; s >>= 1) {
            if (threadIdx.x < s) red[threadIdx.x] += red[threadIdx.x + s];
            __syncthreads();
        }
        if (threadIdx.x == 0) db.p[k][col] = red[0];
        __syncthreads();
    }
}

// clears *flag where the six buffers are not a replicated sharing (party p's
// second share differs from party p+1's first)
__global__ void replicated6_kernel(CSh6<uint64_t> a, size_t n, int *flag) {
    bool ok = true;
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
        ok &= (a.p[1][i] == a.p[2][i]) & (a.p[3][i] == a.p[4][i]) & (a.p[5][i] == a.p[0][i]);
    if (!ok) *flag = 0;
}

// The SGD step of a weight or bias buffer, w -= dividePublic(dw, d)
// (CNNLayer.cu:192-193, FCLayer.cu:211,220), in one pass: dividePublic
// (divide_public_kernel: r = 1, r' = d) leaves the shares [qA, 0, 0, 0, 0, qC],
// so only shares 0 and 5 of w change. dw itself is left undivided.
__global__ void sgd6_kernel(Sh6<uint64_t> w, CSh6<uint64_t> dw, size_t n, uint64_t d, int t) {
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
        const uint64_t s0 = dw.p[0][i] - d, s5 = dw.p[5][i] - d;
        const uint64_t s2 = dw.p[2][i], s4 = dw.p[4][i];
        const uint64_t rA = s0 + dw.p[1][i] + s4;  // party A: own two + C's shareA
        const uint64_t rC = s4 + s5 + s2;          // party C: own two + B's shareA
        w.p[0][i] -= 1 + div_public<uint64_t>(rA, d, t);
        w.p[5][i] -= 1 + div_public<uint64_t>(rC, d, t);
    }
}

__global__ void sub6_kernel(Sh6<uint64_t> a, CSh6<uint64_t> b, size_t n) {
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
#pragma unroll
        for (int k = 0; k < 6; k++) a.p[k][i] -= b.p[k][i];
}

// vectorExpand (matrix.cuh:129-139) of every share: out[j] = in[j / f2]
__global__ void expand6_kernel(CSh6<uint64_t> in, Sh6<uint64_t> out, size_t n_out, int f2) {
    for (size_t j = blockIdx.x * (size_t)blockDim.x + threadIdx.x; j < n_out; j += (size_t)gridDim.x * blockDim.x)
#pragma unroll
        for (int k = 0; k < 6; k++) out.p[k][j] = in.p[k][j / f2];
}

// maxpool_row2im (convolution.cuh:111-152) of every share: window values are
// added into their image positions ((batch, x, y, channel) indexing)
__global__ void row2im6_kernel(CSh6<uint64_t> rows, Sh6<uint64_t> out, int imageHeight, int imageWidth, int f, int Din,
                               int stride, size_t windows) {
    const int wk = (imageWidth - f) / stride + 1, hk = (imageHeight - f) / stride + 1;
    const size_t total = windows * f * f;
    for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < total; e += (size_t)gridDim.x * blockDim.x) {
        const size_t cw = e / (f * f);
        const int v = (int)(e - cw * f * f);
        const size_t per_img = (size_t)wk * hk * Din;
        const size_t b = cw / per_img, rem = cw - b * per_img;
        const int widx = (int)(rem / Din), ch = (int)(rem % Din);
        const int vcol = (widx / hk) * stride + v / f, vrow = (widx % hk) * stride + v % f;
        const size_t o = b * (size_t)imageHeight * imageWidth * Din + (size_t)vcol * imageHeight * Din +
                         (size_t)vrow * Din + ch;
#pragma unroll
        for (int k = 0; k < 6; k++)
            atomicAdd((unsigned long long *)&out.p[k][o], (unsigned long long)rows.p[k][e]);
    }
}

// to_fixed_functor (util/functors.h:117-123) runs on the device in the
// reference: truncation toward zero, saturating, NaN -> 0 (cvt.rzi.u64.f64).
inline uint64_t to_fixed_u64(double x) {
    if (std::isnan(x) || x <= 0.0) return 0;
    if (x >= 18446744073709551616.0) return std::numeric_limits<uint64_t>::max();
    return (uint64_t)x;
}

// The host step of _reveal_softmax_grad (NeuralNetwork.cu:212-254): per party,
// the revealed logits to double, exp, row sums in index order, divide, back to
// fixed point. The reference runs this loop on the host as well. Runs as a
// stream-ordered host function between the reveal's copy-out and the
// softmax's copy-in, so that it can be part of a captured graph.
void CUDART_CB softmax_host(void *arg) {
    pg_net *net = (pg_net *)arg;
    const size_t n = net->tr.n, batch = (size_t)net->tr.batch, classes = n / batch;
    const double scale = (double)(1 << net->tr.fp);
    std::vector<double> fa(n), sums(n / classes);
    for (int p = 0; p < 3; p++) {
        const uint64_t *rev = net->tr.h_rev + p * n;
        uint64_t *sm = net->tr.h_sm + p * n;
        std::fill(sums.begin(), sums.end(), 0.0);
        for (size_t i = 0; i < n; i++) fa[i] = ((double)(int64_t)rev[i]) / scale;
        for (size_t i = 0; i < n; i++) {
            fa[i] = std::exp(fa[i]);
            sums[i / classes] += fa[i];
        }
        for (size_t i = 0; i < n; i++) fa[i] /= sums[i / classes];
        for (size_t i = 0; i < n; i++) sm[i] = to_fixed_u64(fa[i] * scale);
    }
}

unsigned blocks_for(Ctx *c, size_t n) {
    const int sms = c->sm_count > 0 ? c->sm_count : 148;
    size_t b = (n + 255) / 256;
    if (b > (size_t)sms * 8) b = (size_t)sms * 8;
    return (unsigned)(b ? b : 1);
}

template <typename P> CSh6<uint64_t> c6(P const *a) {
    CSh6<uint64_t> r;
    for (int k = 0; k < 6; k++) r.p[k] = a[k];
    return r;
}
Sh6<uint64_t> m6(uint64_t *const *a) {
    Sh6<uint64_t> r;
    for (int k = 0; k < 6; k++) r.p[k] = a[k];
    return r;
}

int sub6(Ctx *c, uint64_t *const *a, const uint64_t *const *b, size_t n) {
    if (!n) return PG_OK;
    sub6_kernel<<<blocks_for(c, n), 256, 0, c->stream>>>(m6(a), c6(b), n);
    c->launches++;
    return launch_status(c, "sub6_kernel");
}

// w -= dividePublic(dw, 2^log_lr), with dividePublic's messages counted
// (rss_divide_public)
int sgd6(Ctx *c, uint64_t *const *w, const uint64_t *const *dw, size_t n, int log_lr) {
    if (n) {
        const uint64_t d = 1ull << log_lr;
        sgd6_kernel<<<blocks_for(c, n), 256, 0, c->stream>>>(m6(w), c6(dw), n, d, pow2_shift<uint64_t>(d));
        c->launches++;
        int st = launch_status(c, "sgd6_kernel");
        if (st) return st;
    }
    comm_msg(c, n * sizeof(uint64_t), n * sizeof(uint64_t));
    comm_round(c);
    return PG_OK;
}

int log_mini_batch(int batch) {  // (int)log2(MINI_BATCH_SIZE), util/model.cu:39
    int t = 0;
    while ((2ll << t) <= batch) t++;
    return t;
}

}  // namespace

// *flag = whether in[]'s six buffers hold a replicated sharing (a set word,
// cleared by the kernel on any mismatch)
static int check_replicated(Ctx *c, const uint64_t *const in[6], size_t n, int *flag) {
    PG_CHECK_CUDA(c, cudaMemsetAsync(flag, 1, sizeof(int), c->stream));
    if (!n) return PG_OK;
    replicated6_kernel<<<blocks_for(c, n), 256, 0, c->stream>>>(c6(in), n, flag);
    c->launches++;
    return launch_status(c, "replicated6_kernel");
}

// Training buffers: per-layer gradients, labels, the softmax step, the
// parameter-gradient scratch, and a parameter snapshot for capture.
static int net_train_setup(pg_net *net) {
    if (net->tr.arena) return PG_OK;
    Ctx *c = net->ctx;
    if (net->fp > 30) return set_error(c, PG_ERR_UNSUPPORTED, "training needs FLOAT_PRECISION <= 30 (got %d)", net->fp);
    if (net->out_n % net->batch) return set_error(c, PG_ERR_SIZE, "output size is not a multiple of the batch");
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    PG_CHECK_CUDA(c, cudaStreamIsCapturing(c->stream, &cs));
    if (cs != cudaStreamCaptureStatusNone)
        return set_error(c, PG_ERR_INVALID_ARG, "training buffers must be set up by an eager step first");
    auto al = [](size_t b) { return (b + 255) & ~(size_t)255; };
    size_t max_w = 0, max_b = 0, max_d = 0, max_sel = 0, params = 0;
    for (auto &L : net->layers) {
        max_w = L.w_n > max_w ? L.w_n : max_w;
        max_b = L.b_n > max_b ? L.b_n : max_b;
        max_d = L.type == PG_LAYER_MAXPOOL && L.d_n > max_d ? L.d_n : max_d;
        const size_t sel = L.type == PG_LAYER_MAXPOOL ? L.d_n : L.type == PG_LAYER_RELU ? L.out_n : 0;
        max_sel = sel > max_sel ? sel : max_sel;
        params += 6 * (al(L.w_n * 8) + al(L.b_n * 8));
    }
    const size_t on = net->out_n;
    size_t bytes = 2 * al(6 * on * 8) + 6 * al(on * 8);  // labels, sdelta, rev[3] + sm[3]
    for (auto &L : net->layers) bytes += al(6 * L.in_n * 8);
    bytes += 6 * (al(max_w * 8) + al(max_b * 8) + al(max_d * 8)) + al(max_sel * 8) + params;
    if (cudaMalloc(&net->tr.arena, bytes) != cudaSuccess) {
        cudaGetLastError();
        net->tr.arena = nullptr;
        return set_error(c, PG_ERR_NO_MEMORY, "training buffers of %zu bytes", bytes);
    }
    if (cudaMallocHost(&net->tr.h_rev, 2 * 3 * on * 8) != cudaSuccess) {
        cudaGetLastError();
        cudaFree(net->tr.arena);
        net->tr.arena = nullptr;
        net->tr.h_rev = nullptr;
        return set_error(c, PG_ERR_NO_MEMORY, "pinned softmax buffers");
    }
    net->tr.h_sm = net->tr.h_rev + 3 * on;
    PG_CHECK_CUDA(c, cudaMemsetAsync(net->tr.arena, 0, bytes, c->stream));
    char *ptr = (char *)net->tr.arena;
    for (int k = 0; k < 6; k++) net->tr.labels[k] = (uint64_t *)(ptr + k * on * 8);
    ptr += al(6 * on * 8);
    for (int k = 0; k < 6; k++) net->tr.sdelta[k] = (uint64_t *)(ptr + k * on * 8);
    ptr += al(6 * on * 8);
    for (int p = 0; p < 3; p++) { net->tr.rev[p] = (uint64_t *)ptr; ptr += al(on * 8); }
    for (int p = 0; p < 3; p++) { net->tr.sm[p] = (uint64_t *)ptr; ptr += al(on * 8); }
    for (auto &L : net->layers) {
        for (int k = 0; k < 6; k++) L.delta[k] = (uint64_t *)(ptr + k * L.in_n * 8);
        ptr += al(6 * L.in_n * 8);
    }
    for (int k = 0; k < 6; k++) { net->tr.dW[k] = (uint64_t *)ptr; ptr += al(max_w * 8); }
    for (int k = 0; k < 6; k++) { net->tr.db[k] = (uint64_t *)ptr; ptr += al(max_b * 8); }
    for (int k = 0; k < 6; k++) { net->tr.pools[k] = (uint64_t *)ptr; ptr += al(max_d * 8); }
    net->tr.zeros = (uint64_t *)ptr;
    ptr += al(max_sel * 8);
    net->tr.backup = (uint64_t *)ptr;
    net->tr.backup_bytes = params;
    net->tr.n = on;
    net->tr.batch = net->batch;
    net->tr.fp = net->fp;
    return PG_OK;
}

// Snapshot / restore of every weight and bias share (device to device).
static int net_params_copy(pg_net *net, bool save) {
    Ctx *c = net->ctx;
    auto al = [](size_t b) { return (b + 255) & ~(size_t)255; };
    char *bk = (char *)net->tr.backup;
    for (auto &L : net->layers)
        for (int k = 0; k < 6; k++) {
            if (L.w_n) {
                PG_CHECK_CUDA(c, cudaMemcpyAsync(save ? (void *)bk : (void *)L.w[k], save ? (void *)L.w[k] : (void *)bk,
                                                 L.w_n * 8, cudaMemcpyDeviceToDevice, c->stream));
            }
            bk += al(L.w_n * 8);
            if (L.b_n) {
                PG_CHECK_CUDA(c, cudaMemcpyAsync(save ? (void *)bk : (void *)L.b[k], save ? (void *)L.b[k] : (void *)bk,
                                                 L.b_n * 8, cudaMemcpyDeviceToDevice, c->stream));
            }
            bk += al(L.b_n * 8);
        }
    if (!save && net->limb_arena)
        for (auto &L : net->layers)
            if (L.packB) {
                int st = lt::run_pack(c, L.plan, (const uint64_t *const *)L.w, L.packB);
                if (st) return st;
            }
    return PG_OK;
}

// _reveal_softmax_grad (NeuralNetwork.cu:207-267) into tr.sdelta.
static int net_softmax_grad(pg_net *net, const uint64_t *const labels[6]) {
    Ctx *c = net->ctx;
    const size_t n = net->out_n;
    NetLayer &last = net->layers.back();
    int st = rss_reconstruct<uint64_t>(c, (const uint64_t *const *)last.out, n, net->tr.rev);
    if (st) return st;
    for (int p = 0; p < 3; p++)
        PG_CHECK_CUDA(c, cudaMemcpyAsync(net->tr.h_rev + p * n, net->tr.rev[p], n * 8, cudaMemcpyDeviceToHost, c->stream));
    PG_CHECK_CUDA(c, cudaLaunchHostFunc(c->stream, softmax_host, net));
    for (int p = 0; p < 3; p++)
        PG_CHECK_CUDA(c, cudaMemcpyAsync(net->tr.sm[p], net->tr.h_sm + p * n, n * 8, cudaMemcpyHostToDevice, c->stream));
    softmax_delta_kernel<<<blocks_for(c, n), 256, 0, c->stream>>>(m6(net->tr.sdelta), net->tr.sm[0], net->tr.sm[2],
                                                                  c6(labels), n);
    c->launches++;
    if ((st = launch_status(c, "softmax_delta_kernel"))) return st;
    const int lmb = log_mini_batch(net->batch);
    if (lmb > 1) st = rss_divide_public<uint64_t>(c, net->tr.sdelta, n, 1ull << lmb, nullptr);
    return st;
}

// The standalone share-GEMM / convolution calls of the backward pass learn
// through the context which of their operands hold a replicated sharing
// (Ctx::rep_a, rep_b), for the limb form's digit images; cleared on return.
struct RepOperands {
    Ctx *c;
    RepOperands(Ctx *c_, bool a, bool b) : c(c_) {
        c->rep_a = a;
        c->rep_b = b;
    }
    ~RepOperands() { c->rep_a = c->rep_b = false; }
};

static int share_gemm(Ctx *c, const uint64_t *const *a, const uint64_t *const *b, uint64_t *const *out, int M, int N,
                      int K, int tA, int tB, int tC, int trunc) {
    if (c->form == PG_FORM_LIMB_TC) return limb3_rss_matmul_u64(c, a, b, out, nullptr, M, N, K, tA, tB, tC, trunc);
    return rss_matmul<uint64_t>(c, a, b, out, nullptr, M, N, K, tA, tB, tC, trunc);
}

static int share_conv(Ctx *c, const uint64_t *const *a, const uint64_t *const *b, uint64_t *const *out, int op,
                      int B, int H, int W, int f, int Din, int Dout, int s, int pd, int trunc) {
    if (c->form == PG_FORM_LIMB_TC) return limb3_rss_conv_u64(c, a, b, out, op, B, H, W, f, Din, Dout, s, pd, trunc);
    return rss_conv<uint64_t>(c, a, b, out, op, B, H, W, f, Din, Dout, s, pd, trunc);
}

// NeuralNetwork::_backward_pass (NeuralNetwork.cu:444-460): every layer's
// backward from the last to the first, each updating its parameters.
static int net_backward(pg_net *net, const uint64_t *const in[6], const uint64_t *const labels[6], int log_lr) {
    Ctx *c = net->ctx;
    if (log_lr < 0 || net->fp + log_lr > 62) return set_error(c, PG_ERR_INVALID_ARG, "bad log learning rate %d", log_lr);
    int st = net_softmax_grad(net, labels);
    if (st) return st;
    const uint64_t *const *din = (const uint64_t *const *)net->tr.sdelta;
    // the softmax delta takes the label shares as given; every FC / CNN
    // input gradient is a replicated sharing ([v, 0, 0, 0, 0, v]), and the
    // ReLU, maxpool and averagepool backward steps keep one replicated
    bool din_rep = false;
    const uint64_t *zeros6[6];
    for (int k = 0; k < 6; k++) zeros6[k] = net->tr.zeros;
    const int B = net->batch;
    for (int li = (int)net->layers.size() - 1; li >= 0; li--) {
        NetLayer &L = net->layers[li];
        const uint64_t *const *fwd_in = li ? (const uint64_t *const *)net->layers[li - 1].out : in;
        const bool fwd_rep = li ? net->layers[li - 1].out_rep : false;
        switch (L.type) {
            case PG_LAYER_FC: {  // FCLayer::backward (FCLayer.cu:132-217)
                const int din_ = L.p[0], dout = L.p[1];
                {
                    RepOperands rep(c, din_rep, fwd_rep);  // both GEMMs take the delta as their image operand
                    if ((st = share_gemm(c, din, (const uint64_t *const *)L.w, L.delta, B, din_, dout, 1, 0, 1, net->fp)))
                        return st;
                    if ((st = share_gemm(c, din, fwd_in, net->tr.dW, dout, din_, B, 0, 1, 0, net->fp + log_lr)))
                        return st;
                }
                if ((st = sub6(c, L.w, net->tr.dW, L.w_n))) return st;
                {
                    // reduceSum(delta, db, false, outputDim, batchSize) into a zeroed db, as the
                    // reference calls it, for the six shares at once
                    const int blocks = 6 * dout < 4096 ? 6 * dout : 4096;
                    bias_grad6_kernel<<<blocks, 256, 0, c->stream>>>(c6(din), m6(net->tr.db), dout, B);
                    c->launches++;
                    if ((st = launch_status(c, "bias_grad6_kernel"))) return st;
                }
                if ((st = sgd6(c, L.b, net->tr.db, L.b_n, log_lr))) return st;
                break;
            }
            case PG_LAYER_CNN: {  // CNNLayer::backward (CNNLayer.cu:114-193)
                const int H = L.p[0], W = L.p[1], Din = L.p[2], Dout = L.p[3], f = L.p[4], s = L.p[5], pd = L.p[6];
                {
                    // the input gradient's image is dY; the weight gradient's the forward input
                    RepOperands rep(c, din_rep, fwd_rep);
                    if ((st = share_conv(c, din, (const uint64_t *const *)L.w, L.delta, PG_CONV_DGRAD, B, H, W, f, Din,
                                         Dout, s, pd, net->fp)))
                        return st;
                    if ((st = share_conv(c, din, fwd_in, net->tr.dW, PG_CONV_WGRAD, B, H, W, f, Din, Dout, s, pd,
                                         net->fp)))
                        return st;
                }
                if ((st = sgd6(c, L.w, net->tr.dW, L.w_n, log_lr))) return st;
                break;
            }
            case PG_LAYER_RELU:  // ReLULayer::backward (ReLULayer.cu:90-124)
                st = rss_select<uint64_t, uint8_t>(c, zeros6, din, (const uint8_t *const *)L.d, L.delta, L.in_n);
                if (st) return st;
                break;
            case PG_LAYER_MAXPOOL: {  // MaxpoolLayer::backward (MaxpoolLayer.cu:133-185)
                const int H = L.p[0], W = L.p[1], C = L.p[2], f = L.p[3], s = L.p[4];
                expand6_kernel<<<blocks_for(c, L.d_n), 256, 0, c->stream>>>(c6(din), m6(net->tr.pools), L.d_n, f * f);
                c->launches++;
                if ((st = launch_status(c, "expand6_kernel"))) return st;
                st = rss_select<uint64_t, uint8_t>(c, zeros6, (const uint64_t *const *)net->tr.pools,
                                                   (const uint8_t *const *)L.d, net->tr.pools, L.d_n);
                if (st) return st;
                PG_CHECK_CUDA(c, cudaMemsetAsync(L.delta[0], 0, 6 * L.in_n * 8, c->stream));
                // row2im gets (imageWidth, imageHeight) in its (imageHeight, imageWidth) slots, as the reference passes them
                const size_t windows = L.d_n / ((size_t)f * f);
                row2im6_kernel<<<blocks_for(c, L.d_n), 256, 0, c->stream>>>(
                    c6(net->tr.pools), m6(L.delta), W, H, f, C, s, windows);
                c->launches++;
                if ((st = launch_status(c, "row2im6_kernel"))) return st;
                break;
            }
            case PG_LAYER_AVGPOOL:  // AveragepoolLayer::backward (AveragepoolLayer.cu:88-117)
                st = rss_avgpool_backward<uint64_t>(c, din, L.delta, L.p[0], L.p[1], L.p[2], L.p[3], L.p[4], B);
                if (st) return st;
                break;
            default: return set_error(c, PG_ERR_INVALID_ARG, "bad layer type %d", L.type);
        }
        // the limb form keeps packed weights: repack the updated ones
        if (net->limb_arena && L.packB && (st = lt::run_pack(c, L.plan, (const uint64_t *const *)L.w, L.packB))) return st;
        din = (const uint64_t *const *)L.delta;
        if (L.type == PG_LAYER_FC || L.type == PG_LAYER_CNN) din_rep = true;
    }
    return PG_OK;
}

static int net_train(pg_net *net, const uint64_t *const in[6], const uint64_t *const labels[6], int log_lr) {
    int st = net_run(net, in);
    if (st) return st;
    return net_backward(net, in, labels, log_lr);
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
            case PG_LAYER_MAXPOOL:
            case PG_LAYER_AVGPOOL: {
                int H = L.p[0], W = L.p[1], C = L.p[2], f = L.p[3], s = L.p[4];
                if (f <= 0 || s <= 0 || f > H || f > W) {
                    delete net;
                    return set_error(c, PG_ERR_SIZE, "layer %d: bad pool geometry", i);
                }
                L.in_n = (size_t)batch * H * W * C;
                L.out_n = (size_t)batch * ((H - f) / s + 1) * ((W - f) / s + 1) * C;
                L.d_n = L.type == PG_LAYER_MAXPOOL ? L.out_n * f * f : 0;
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

// Work enqueued on the context stream that reads (or writes) the first input
// buffer set: pg_net_forward_host's next copy into it waits for that.
static void mark_in_used(pg_net *net) {
    if (net->in_free[0]) cudaEventRecord(net->in_free[0], net->ctx->stream);
}

// the captured forward (both input buffer sets' graphs)
static void drop_forward_graphs(pg_net *net) {
    if (net->exec) cudaGraphExecDestroy(net->exec);
    if (net->graph) cudaGraphDestroy(net->graph);
    if (net->exec_alt) cudaGraphExecDestroy(net->exec_alt);
    if (net->graph_alt) cudaGraphDestroy(net->graph_alt);
    net->exec = net->exec_alt = nullptr;
    net->graph = net->graph_alt = nullptr;
}

int pg_net_destroy(pg_net *net) {
    if (!net) return PG_ERR_INVALID_ARG;
    for (auto e : net->ev) cudaEventDestroy(e);
    if (net->copy) cudaStreamSynchronize(net->copy);
    drop_forward_graphs(net);
    for (int s = 0; s < 2; s++) {
        if (net->in_ready[s]) cudaEventDestroy(net->in_ready[s]);
        if (net->in_free[s]) cudaEventDestroy(net->in_free[s]);
    }
    if (net->copy) cudaStreamDestroy(net->copy);
    if (net->exec_train) cudaGraphExecDestroy(net->exec_train);
    if (net->graph_train) cudaGraphDestroy(net->graph_train);
    if (net->arena || net->limb_arena || net->tr.arena) cudaStreamSynchronize(net->ctx->stream);
    if (net->arena) cudaFree(net->arena);
    if (net->limb_arena) cudaFree(net->limb_arena);
    if (net->tr.arena) cudaFree(net->tr.arena);
    if (net->tr.h_rev) cudaFreeHost(net->tr.h_rev);
    if (net->in_alt) cudaFree(net->in_alt);
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
    if (L.b_n && bias) {
        for (int k = 0; k < 6; k++)
            PG_CHECK_CUDA(c, cudaMemcpyAsync(L.b[k], bias[k], L.b_n * 8, cudaMemcpyDeviceToDevice, c->stream));
        // whether the layer's outputs stay a replicated sharing: party p's
        // second bias share equals party p+1's first
        std::vector<uint64_t> hb(6 * L.b_n);
        for (int k = 0; k < 6; k++)
            PG_CHECK_CUDA(c, cudaMemcpyAsync(hb.data() + k * L.b_n, bias[k], L.b_n * 8, cudaMemcpyDeviceToHost,
                                             c->stream));
        PG_CHECK_CUDA(c, cudaStreamSynchronize(c->stream));
        bool rep = true;
        for (int p = 0; p < 3 && rep; p++)
            rep = memcmp(hb.data() + (2 * p + 1) * L.b_n, hb.data() + ((2 * p + 2) % 6) * L.b_n, L.b_n * 8) == 0;
        if (rep != L.b_replicated) {
            // captured steps chose their image layouts with the old flag
            if (net->copy) cudaStreamSynchronize(net->copy);
            drop_forward_graphs(net);
            if (net->exec_train) cudaGraphExecDestroy(net->exec_train);
            if (net->graph_train) cudaGraphDestroy(net->graph_train);
            net->exec_train = nullptr;
            net->graph_train = nullptr;
        }
        L.b_replicated = rep;
    }
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
    mark_in_used(net);
    if (st) return st;
    NetLayer &last = net->layers.back();
    for (int k = 0; k < 6; k++)
        if (out[k] != last.out[k])
            PG_CHECK_CUDA(c, cudaMemcpyAsync(out[k], last.out[k], net->out_n * 8, cudaMemcpyDeviceToDevice, c->stream));
    return PG_OK;
}

// One forward captured as a graph reading the input buffers in[] (replays go
// to the context stream); its accounting goes to comm_per_fwd /
// launches_per_fwd.
static int capture_forward(pg_net *net, const uint64_t *const in[6], cudaGraph_t &graph, cudaGraphExec_t &exec) {
    Ctx *c = net->ctx;
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
    int st = e0 == cudaSuccess ? net_run(net, in) : PG_ERR_CUDA;
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
    graph = g;
    PG_CHECK_CUDA(c, cudaGraphInstantiate(&exec, g, 0));
    net->launches_per_fwd = launched;  // capture does not execute: replays add these
    return PG_OK;
}

int pg_net_capture(pg_net *net) {
    if (!net) return PG_ERR_INVALID_ARG;
    Ctx *c = net->ctx;
    if (net->copy) PG_CHECK_CUDA(c, cudaStreamSynchronize(net->copy));
    drop_forward_graphs(net);
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
    int st = capture_forward(net, (const uint64_t *const *)net->in, net->graph, net->exec);
    if (st) return st;
    net->fwd_graph_held = net->last_fwd_held;  // the captured forward's kind
    // the second input buffer set of pg_net_forward_host and its graph; without
    // them (no memory) the host forward replays the first graph
    if (!net->in_alt && cudaMalloc(&net->in_alt, 6 * net->in_n * 8) != cudaSuccess) {
        cudaGetLastError();
        net->in_alt = nullptr;
    }
    if (net->in_alt && !net->copy) {
        if (cudaStreamCreateWithFlags(&net->copy, cudaStreamNonBlocking) != cudaSuccess) {
            cudaGetLastError();
            net->copy = nullptr;
        }
        for (int s = 0; s < 2 && net->copy; s++)
            if (cudaEventCreateWithFlags(&net->in_ready[s], cudaEventDisableTiming) != cudaSuccess ||
                cudaEventCreateWithFlags(&net->in_free[s], cudaEventDisableTiming) != cudaSuccess)
                return set_error(c, PG_ERR_CUDA, "cudaEventCreate failed");
    }
    if (net->in_alt && net->copy) {
        const uint64_t *alt[6];
        for (int k = 0; k < 6; k++) alt[k] = net->in_alt + (size_t)k * net->in_n;
        if ((st = capture_forward(net, alt, net->graph_alt, net->exec_alt))) return st;
    }
    net->slot = 0;
    return PG_OK;
}

static int net_replay_or_run(pg_net *net) {
    Ctx *c = net->ctx;
    if (net->exec) {
        PG_CHECK_CUDA(c, cudaGraphLaunch(net->exec, c->stream));
        for (int k = 0; k < 9; k++) c->comm[k] += net->comm_per_fwd[k];
        c->launches += net->launches_per_fwd;
        net->last_fwd_held = net->fwd_graph_held;
        mark_in_used(net);
        return PG_OK;
    }
    int st = net_run(net, (const uint64_t *const *)net->in);
    mark_in_used(net);
    return st;
}

int pg_net_forward_host(pg_net *net, const uint64_t *in_host, uint64_t *out_host) {
    if (!net || !in_host || !out_host) return PG_ERR_INVALID_ARG;
    Ctx *c = net->ctx;
    if (net->exec && net->exec_alt) {
        // Double-buffered: this call's input goes to one buffer set on the
        // copy stream (once the replay that last read it has finished) while
        // the previous call's replay still runs on the context stream.
        const int s = net->slot;
        net->slot ^= 1;
        uint64_t *buf = s ? net->in_alt : net->in[0];
        PG_CHECK_CUDA(c, cudaStreamWaitEvent(net->copy, net->in_free[s], 0));
        PG_CHECK_CUDA(c, cudaMemcpyAsync(buf, in_host, 6 * net->in_n * 8, cudaMemcpyHostToDevice, net->copy));
        PG_CHECK_CUDA(c, cudaEventRecord(net->in_ready[s], net->copy));
        PG_CHECK_CUDA(c, cudaStreamWaitEvent(c->stream, net->in_ready[s], 0));
        PG_CHECK_CUDA(c, cudaGraphLaunch(s ? net->exec_alt : net->exec, c->stream));
        for (int k = 0; k < 9; k++) c->comm[k] += net->comm_per_fwd[k];
        c->launches += net->launches_per_fwd;
        net->last_fwd_held = net->fwd_graph_held;
        PG_CHECK_CUDA(c, cudaEventRecord(net->in_free[s], c->stream));
        NetLayer &last = net->layers.back();
        PG_CHECK_CUDA(c, cudaMemcpyAsync(out_host, last.out[0], 6 * net->out_n * 8, cudaMemcpyDeviceToHost, c->stream));
        return PG_OK;
    }
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
    if (L.out_held && net->last_fwd_held && (size_t)layer + 1 < net->layers.size()) {
        // the last (inference) forward kept this ReLU output in the next
        // layer's digit image alone: rebuild the six shares from it
        Ctx *c = net->ctx;
        NetLayer &nx = net->layers[layer + 1];
        int st = lt::run_image_decode(c, nx.plan, nx.held, L.out_n, L.out, nx.held_shared);
        if (st) return st;
        PG_CHECK_CUDA(c, cudaStreamSynchronize(c->stream));
    }
    if (out)
        for (int k = 0; k < 6; k++) ((uint64_t **)out)[k] = L.out[k];
    if (n) *n = L.out_n;
    return PG_OK;
}

int pg_net_layer_plan(pg_net *net, int layer, int out[4]) {
    if (!net || !out || layer < 0 || layer >= (int)net->layers.size()) return PG_ERR_INVALID_ARG;
    NetLayer &L = net->layers[layer];
    for (int k = 0; k < 4; k++) out[k] = 0;
    if ((L.type == PG_LAYER_FC || L.type == PG_LAYER_CNN) && net->limb_arena) {
        out[0] = L.u64 ? 2 : 1;
        out[1] = L.plan.posmajor;
        out[2] = L.split;
        out[3] = L.plan.tiles_m * L.plan.ntiles_n;
    } else if (L.type == PG_LAYER_FC || L.type == PG_LAYER_CNN) {
        out[0] = 2;
    }
    return PG_OK;
}

// ----------------------------------------------------------- training API

int pg_net_train_setup(pg_net *net) {
    if (!net) return PG_ERR_INVALID_ARG;
    return net_train_setup(net);
}

int pg_net_label_shares(pg_net *net, uint64_t *out[6]) {
    if (!net || !out) return PG_ERR_INVALID_ARG;
    int st = net_train_setup(net);
    if (st) return st;
    for (int k = 0; k < 6; k++) out[k] = net->tr.labels[k];
    return PG_OK;
}

int pg_net_backward(pg_net *net, const uint64_t *const in[6], const uint64_t *const labels[6], int log_lr) {
    if (!net || !in || !labels) return PG_ERR_INVALID_ARG;
    // the backward reads the forward's bit shares and layer outputs, which an
    // inference forward does not keep
    if (net->last_fwd_held)
        return set_error(net->ctx, PG_ERR_INVALID_ARG,
                         "the last forward was an inference forward: call pg_net_train_setup before the forward");
    int st = net_train_setup(net);
    if (st) return st;
    return net_backward(net, in, labels, log_lr);
}

int pg_net_train_step(pg_net *net, const uint64_t *const in[6], const uint64_t *const labels[6], int log_lr) {
    if (!net || !in || !labels) return PG_ERR_INVALID_ARG;
    int st = net_train_setup(net);
    if (st) return st;
    return net_train(net, in, labels, log_lr);
}

int pg_net_capture_train(pg_net *net, int log_lr) {
    if (!net) return PG_ERR_INVALID_ARG;
    Ctx *c = net->ctx;
    int st = net_train_setup(net);
    if (st) return st;
    if (net->exec_train) {
        cudaGraphExecDestroy(net->exec_train);
        net->exec_train = nullptr;
    }
    if (net->graph_train) {
        cudaGraphDestroy(net->graph_train);
        net->graph_train = nullptr;
    }
    const uint64_t *const *in = (const uint64_t *const *)net->in;
    const uint64_t *const *lab = (const uint64_t *const *)net->tr.labels;
    // One eager step first (it sizes the context scratch and sets up the
    // limb-form buffers), with the parameters restored afterwards.
    {
        uint64_t comm_save[9];
        memcpy(comm_save, c->comm, sizeof(comm_save));
        uint64_t launches_save = c->launches.load();
        int st0 = net_params_copy(net, true);
        if (!st0) st0 = net_train(net, in, lab, log_lr);
        if (!st0) st0 = net_params_copy(net, false);
        memcpy(c->comm, comm_save, sizeof(comm_save));
        c->launches = launches_save;
        if (st0) return st0;
        PG_CHECK_CUDA(c, cudaStreamSynchronize(c->stream));
    }
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
    st = e0 == cudaSuccess ? net_train(net, in, lab, log_lr) : PG_ERR_CUDA;
    cudaGraph_t g = nullptr;
    cudaError_t e = e0 == cudaSuccess ? cudaStreamEndCapture(cap, &g) : e0;
    c->stream = user;
    cudaStreamSynchronize(cap);
    cudaStreamDestroy(cap);
    cudaEventDestroy(ev);
    for (int k = 0; k < 9; k++) net->comm_per_train[k] = c->comm[k] - comm_before[k];
    memcpy(c->comm, comm_before, sizeof(comm_before));
    uint64_t launched = c->launches.load() - launches_before;
    c->launches = launches_before;
    if (st) {
        if (g) cudaGraphDestroy(g);
        return st;
    }
    if (e != cudaSuccess) return set_error(c, PG_ERR_CUDA, "graph capture: %s", cudaGetErrorString(e));
    net->graph_train = g;
    PG_CHECK_CUDA(c, cudaGraphInstantiate(&net->exec_train, g, 0));
    net->launches_per_train = launched;
    return PG_OK;
}

int pg_net_train_resident(pg_net *net) {
    if (!net) return PG_ERR_INVALID_ARG;
    Ctx *c = net->ctx;
    if (!net->exec_train) return set_error(c, PG_ERR_INVALID_ARG, "no captured training step");
    PG_CHECK_CUDA(c, cudaGraphLaunch(net->exec_train, c->stream));
    for (int k = 0; k < 9; k++) c->comm[k] += net->comm_per_train[k];
    c->launches += net->launches_per_train;
    net->last_fwd_held = false;
    mark_in_used(net);
    return PG_OK;
}

int pg_net_train_host(pg_net *net, const uint64_t *in_host, const uint64_t *labels_host, uint64_t *out_host,
                      int log_lr) {
    if (!net || !in_host || !labels_host || !out_host) return PG_ERR_INVALID_ARG;
    Ctx *c = net->ctx;
    int st = net_train_setup(net);
    if (st) return st;
    PG_CHECK_CUDA(c, cudaMemcpyAsync(net->in[0], in_host, 6 * net->in_n * 8, cudaMemcpyHostToDevice, c->stream));
    PG_CHECK_CUDA(c, cudaMemcpyAsync(net->tr.labels[0], labels_host, 6 * net->out_n * 8, cudaMemcpyHostToDevice,
                                     c->stream));
    st = net->exec_train ? pg_net_train_resident(net)
                         : net_train(net, (const uint64_t *const *)net->in, (const uint64_t *const *)net->tr.labels,
                                     log_lr);
    mark_in_used(net);
    if (st) return st;
    NetLayer &last = net->layers.back();
    PG_CHECK_CUDA(c, cudaMemcpyAsync(out_host, last.out[0], 6 * net->out_n * 8, cudaMemcpyDeviceToHost, c->stream));
    return PG_OK;
}

int pg_net_layer_delta(pg_net *net, int layer, uint64_t *out[6], size_t *n) {
    if (!net || !out || layer < -1 || layer >= (int)net->layers.size()) return PG_ERR_INVALID_ARG;
    if (!net->tr.arena) return set_error(net->ctx, PG_ERR_INVALID_ARG, "no training step has run");
    // layer -1: the softmax gradient that enters the last layer
    for (int k = 0; k < 6; k++) out[k] = layer < 0 ? net->tr.sdelta[k] : net->layers[layer].delta[k];
    if (n) *n = layer < 0 ? net->out_n : net->layers[layer].in_n;
    return PG_OK;
}

int pg_net_layer_params(pg_net *net, int layer, uint64_t *w[6], uint64_t *b[6], size_t *w_n, size_t *b_n) {
    if (!net || layer < 0 || layer >= (int)net->layers.size()) return PG_ERR_INVALID_ARG;
    NetLayer &L = net->layers[layer];
    for (int k = 0; k < 6; k++) {
        if (w) w[k] = L.w_n ? L.w[k] : nullptr;
        if (b) b[k] = L.b_n ? L.b[k] : nullptr;
    }
    if (w_n) *w_n = L.w_n;
    if (b_n) *b_n = L.b_n;
    return PG_OK;
}

}  // extern "C"
