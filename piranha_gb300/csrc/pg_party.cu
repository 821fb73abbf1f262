// pg_party.cu — party mode: one RSS party per process, messages over TCP in
// the reference's wire format (src/util/basicSockets.cpp, src/util/connect.cu,
// src/gpu/DeviceData.h:87-129), local arithmetic on the GPU.
//
// Wire format, kept identical so that a reference party can be a peer: for
// every ordered pair (sender s, receiver r) the receiver listens on
// base + s * n + r and the sender opens three TCP connections to it
// (NUMCONNECTIONS); a message is the raw bytes of the vector on connection 0,
// with no header or length. Connections are made in the reference's serial
// order: for each other party i, a lower-numbered i is connected to first and
// then listened for, a higher-numbered one the other way round.
//
// What is added: every wait is bounded (connect, accept, send, receive) and
// turns into a status; a peer that closes mid-message is an error, not a
// zero-filled buffer; the end-of-step check swaps byte counters on
// connection 1 and looks for unread bytes on connection 0; and a host-side
// fault injector (drop / duplicate / truncate the nth send) tests that
// detection.
#include <arpa/inet.h>
#include <errno.h>
#include <fcntl.h>
#include <netdb.h>
#include <netinet/in.h>
#include <netinet/tcp.h>
#include <poll.h>
#include <sys/socket.h>
#include <time.h>
#include <unistd.h>

#include <cstring>
#include <string>
#include <thread>
#include <vector>

#include "pg_common.cuh"

namespace pg {
template <typename T> int plain_gemm(Ctx *, int, int, int, const T *, int, const T *, int, T *, int);
void *scratch(Ctx *c, size_t bytes);
}  // namespace pg

using namespace pg;

namespace {

constexpr int kConns = 3;     // connections per ordered pair of parties (NUMCONNECTIONS)
constexpr int kMaxParties = 8;

uint64_t now_ms() {
    timespec ts;
    clock_gettime(CLOCK_MONOTONIC, &ts);
    return (uint64_t)ts.tv_sec * 1000 + (uint64_t)ts.tv_nsec / 1000000;
}

}  // namespace

struct pg_party {
    int party = 0, n = 0;
    int timeout_ms = 10000;
    int base_port = 32000;
    std::vector<std::string> hosts;
    int snd[kMaxParties][kConns];  // to party i
    int rcv[kMaxParties][kConns];  // from party i
    uint64_t tx[kMaxParties] = {0}, rx[kMaxParties] = {0};
    uint64_t rounds = 0;
    int fault = PG_FAULT_NONE, fault_countdown = 0;
    std::string err;
    void *stage_out = nullptr, *stage_in = nullptr;  // pinned host staging of device messages
    size_t stage_out_bytes = 0, stage_in_bytes = 0;

    pg_party() {
        for (int i = 0; i < kMaxParties; i++)
            for (int k = 0; k < kConns; k++) snd[i][k] = rcv[i][k] = -1;
    }
    int fail(int code, const char *fmt, ...) {
        char buf[512];
        va_list ap;
        va_start(ap, fmt);
        vsnprintf(buf, sizeof(buf), fmt, ap);
        va_end(ap);
        err = buf;
        return code;
    }
};

namespace {

void set_nodelay(int fd) {
    int one = 1;
    setsockopt(fd, IPPROTO_TCP, TCP_NODELAY, &one, sizeof(one));
}

// Accept kConns connections on port (bounded by the deadline).
int listen_for(pg_party *p, int peer, int port, uint64_t deadline) {
    int srv = socket(AF_INET, SOCK_STREAM, 0);
    if (srv < 0) return p->fail(PG_ERR_COMM, "socket: %s", strerror(errno));
    int one = 1;
    setsockopt(srv, SOL_SOCKET, SO_REUSEADDR, &one, sizeof(one));
    sockaddr_in addr;
    memset(&addr, 0, sizeof(addr));
    addr.sin_family = AF_INET;
    addr.sin_addr.s_addr = htonl(INADDR_ANY);
    addr.sin_port = htons((uint16_t)port);
    while (bind(srv, (sockaddr *)&addr, sizeof(addr)) < 0) {
        if (now_ms() > deadline) {
            close(srv);
            return p->fail(PG_ERR_TIMEOUT, "bind to port %d: %s", port, strerror(errno));
        }
        usleep(50000);
    }
    listen(srv, 16);
    for (int k = 0; k < kConns; k++) {
        pollfd pf = {srv, POLLIN, 0};
        const uint64_t t = now_ms();
        const int left = t < deadline ? (int)(deadline - t) : 0;
        if (poll(&pf, 1, left) <= 0) {
            close(srv);
            return p->fail(PG_ERR_TIMEOUT, "party %d did not connect to port %d", peer, port);
        }
        const int fd = accept(srv, nullptr, nullptr);
        if (fd < 0) {
            close(srv);
            return p->fail(PG_ERR_COMM, "accept on port %d: %s", port, strerror(errno));
        }
        set_nodelay(fd);
        p->rcv[peer][k] = fd;
    }
    close(srv);
    return PG_OK;
}

// Open kConns connections to host:port, retrying until the deadline.
int connect_to(pg_party *p, int peer, const char *host, int port, uint64_t deadline) {
    addrinfo hints, *res = nullptr;
    memset(&hints, 0, sizeof(hints));
    hints.ai_family = AF_INET;
    hints.ai_socktype = SOCK_STREAM;
    char ports[16];
    snprintf(ports, sizeof(ports), "%d", port);
    if (getaddrinfo(host, ports, &hints, &res) != 0 || !res)
        return p->fail(PG_ERR_INVALID_ARG, "cannot resolve %s", host);
    for (int k = 0; k < kConns; k++) {
        for (;;) {
            const int fd = socket(AF_INET, SOCK_STREAM, 0);
            if (fd < 0) {
                freeaddrinfo(res);
                return p->fail(PG_ERR_COMM, "socket: %s", strerror(errno));
            }
            if (connect(fd, res->ai_addr, res->ai_addrlen) == 0) {
                set_nodelay(fd);
                p->snd[peer][k] = fd;
                break;
            }
            close(fd);
            if (now_ms() > deadline) {
                freeaddrinfo(res);
                return p->fail(PG_ERR_TIMEOUT, "party %d (%s:%d) is not listening", peer, host, port);
            }
            usleep(20000);
        }
    }
    freeaddrinfo(res);
    return PG_OK;
}

int fail_to(std::string &err, int code, const char *fmt, ...) {
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof(buf), fmt, ap);
    va_end(ap);
    err = buf;
    return code;
}

// write all bytes (bounded by the deadline)
int write_all(std::string &err, int fd, const uint8_t *data, size_t bytes, uint64_t deadline) {
    size_t done = 0;
    while (done < bytes) {
        pollfd pf = {fd, POLLOUT, 0};
        const uint64_t t = now_ms();
        const int left = t < deadline ? (int)(deadline - t) : 0;
        if (poll(&pf, 1, left) <= 0) return fail_to(err, PG_ERR_TIMEOUT, "send stalled after %zu of %zu bytes", done, bytes);
        const ssize_t w = send(fd, data + done, bytes - done, MSG_NOSIGNAL);
        if (w < 0) {
            if (errno == EINTR || errno == EAGAIN) continue;
            return fail_to(err, PG_ERR_COMM, "send: %s", strerror(errno));
        }
        done += (size_t)w;
    }
    return PG_OK;
}

// read exactly bytes (bounded by the deadline)
int read_all(std::string &err, int fd, uint8_t *data, size_t bytes, uint64_t deadline, int peer) {
    size_t done = 0;
    while (done < bytes) {
        pollfd pf = {fd, POLLIN, 0};
        const uint64_t t = now_ms();
        const int left = t < deadline ? (int)(deadline - t) : 0;
        if (poll(&pf, 1, left) <= 0)
            return fail_to(err, PG_ERR_TIMEOUT, "message from party %d stopped after %zu of %zu bytes", peer, done,
                           bytes);
        const ssize_t r = recv(fd, data + done, bytes - done, 0);
        if (r == 0)
            return fail_to(err, PG_ERR_COMM, "party %d closed the connection after %zu of %zu bytes", peer, done, bytes);
        if (r < 0) {
            if (errno == EINTR || errno == EAGAIN) continue;
            return fail_to(err, PG_ERR_COMM, "recv: %s", strerror(errno));
        }
        done += (size_t)r;
    }
    return PG_OK;
}

}  // namespace

// ------------------------------------------------------------- C ABI: transport

namespace {

// the message of this thread's last failed pg_party_create (pg_party_last_error(NULL))
std::string &create_error() {
    static thread_local std::string e;
    return e;
}

// one data message on connection 0, through the fault injector (err: the
// calling thread's error text)
int party_send(pg_party *p, int to, const void *data, size_t bytes, std::string &err) {
    if (to < 0 || to >= p->n || to == p->party) return fail_to(err, PG_ERR_INVALID_ARG, "bad destination party %d", to);
    if (bytes && !data) return fail_to(err, PG_ERR_INVALID_ARG, "null data");
    int fault = PG_FAULT_NONE;
    if (p->fault != PG_FAULT_NONE && --p->fault_countdown == 0) {
        fault = p->fault;
        p->fault = PG_FAULT_NONE;
    }
    p->tx[to] += bytes;  // what the sender believes it sent (comm_profiler.add_comm_bytes)
    if (fault == PG_FAULT_DROP) return PG_OK;
    const uint64_t deadline = now_ms() + (uint64_t)p->timeout_ms;
    const size_t w = fault == PG_FAULT_TRUNCATE ? bytes / 2 : bytes;
    int st = write_all(err, p->snd[to][0], (const uint8_t *)data, w, deadline);
    if (!st && fault == PG_FAULT_DUPLICATE) st = write_all(err, p->snd[to][0], (const uint8_t *)data, bytes, deadline);
    return st;
}

int party_recv(pg_party *p, int from, void *data, size_t bytes, std::string &err) {
    if (from < 0 || from >= p->n || from == p->party) return fail_to(err, PG_ERR_INVALID_ARG, "bad source party %d", from);
    if (bytes && !data) return fail_to(err, PG_ERR_INVALID_ARG, "null data");
    int st = read_all(err, p->rcv[from][0], (uint8_t *)data, bytes, now_ms() + (uint64_t)p->timeout_ms, from);
    if (!st) p->rx[from] += bytes;
    return st;
}

}  // namespace

extern "C" {

int pg_party_create(pg_party **out, int party, int num_parties, const char *const *hosts, int base_port,
                    int timeout_ms) {
    if (!out) return PG_ERR_INVALID_ARG;
    *out = nullptr;
    if (num_parties < 2 || num_parties > kMaxParties || party < 0 || party >= num_parties || !hosts ||
        base_port <= 0 || base_port + num_parties * num_parties > 65535 || timeout_ms <= 0)
        return PG_ERR_INVALID_ARG;
    pg_party *p = new pg_party();
    p->party = party;
    p->n = num_parties;
    p->timeout_ms = timeout_ms;
    p->base_port = base_port;
    for (int i = 0; i < num_parties; i++) p->hosts.push_back(hosts[i] ? hosts[i] : "127.0.0.1");
    const uint64_t deadline = now_ms() + (uint64_t)timeout_ms;
    int st = PG_OK;
    // initializeCommunicationSerial (connect.cu:64-80): the receiving party
    // listens on base + sender * n + receiver
    for (int i = 0; i < num_parties && !st; i++) {
        if (i == party) continue;
        const int listen_port = base_port + i * num_parties + party;
        const int connect_port = base_port + party * num_parties + i;
        if (i < party) {
            st = connect_to(p, i, p->hosts[i].c_str(), connect_port, deadline);
            if (!st) st = listen_for(p, i, listen_port, deadline);
        } else {
            st = listen_for(p, i, listen_port, deadline);
            if (!st) st = connect_to(p, i, p->hosts[i].c_str(), connect_port, deadline);
        }
    }
    if (st) {
        create_error() = p->err;
        pg_party_destroy(p);
        return st;
    }
    *out = p;
    return PG_OK;
}

int pg_party_destroy(pg_party *p) {
    if (!p) return PG_ERR_INVALID_ARG;
    for (int i = 0; i < kMaxParties; i++)
        for (int k = 0; k < kConns; k++) {
            if (p->snd[i][k] >= 0) close(p->snd[i][k]);
            if (p->rcv[i][k] >= 0) close(p->rcv[i][k]);
        }
    if (p->stage_out) cudaFreeHost(p->stage_out);
    if (p->stage_in) cudaFreeHost(p->stage_in);
    delete p;
    return PG_OK;
}

const char *pg_party_last_error(pg_party *p) { return p ? p->err.c_str() : create_error().c_str(); }

int pg_party_send(pg_party *p, int to, const void *data, size_t bytes) {
    return p ? party_send(p, to, data, bytes, p->err) : PG_ERR_INVALID_ARG;
}

int pg_party_recv(pg_party *p, int from, void *data, size_t bytes) {
    return p ? party_recv(p, from, data, bytes, p->err) : PG_ERR_INVALID_ARG;
}

int pg_party_counters(pg_party *p, uint64_t *out) {
    if (!p || !out) return PG_ERR_INVALID_ARG;
    for (int i = 0; i < p->n; i++) {
        out[i] = p->tx[i];
        out[p->n + i] = p->rx[i];
    }
    out[2 * p->n] = p->rounds;
    return PG_OK;
}

int pg_party_inject(pg_party *p, int kind, int nth) {
    if (!p) return PG_ERR_INVALID_ARG;
    if (kind < PG_FAULT_NONE || kind > PG_FAULT_TRUNCATE || (kind != PG_FAULT_NONE && nth < 1))
        return p->fail(PG_ERR_INVALID_ARG, "fault %d at send %d", kind, nth);
    p->fault = kind;
    p->fault_countdown = nth;
    return PG_OK;
}

int pg_party_check(pg_party *p) {
    if (!p) return PG_ERR_INVALID_ARG;
    const uint64_t deadline = now_ms() + (uint64_t)p->timeout_ms;
    int first = PG_OK;
    std::string first_err;
    // every pair swaps (sent to the peer, received from the peer) on
    // connection 1, the lower-numbered party of a pair writing first; all
    // pairs are swapped before any verdict, so every party finishes the check
    for (int i = 0; i < p->n; i++) {
        if (i == p->party) continue;
        const uint64_t mine[2] = {p->tx[i], p->rx[i]};
        uint64_t theirs[2] = {0, 0};
        std::string e;
        int st;
        if (p->party < i) {
            st = write_all(e, p->snd[i][1], (const uint8_t *)mine, sizeof(mine), deadline);
            if (!st) st = read_all(e, p->rcv[i][1], (uint8_t *)theirs, sizeof(theirs), deadline, i);
        } else {
            st = read_all(e, p->rcv[i][1], (uint8_t *)theirs, sizeof(theirs), deadline, i);
            if (!st) st = write_all(e, p->snd[i][1], (const uint8_t *)mine, sizeof(mine), deadline);
        }
        if (!st && (theirs[0] != mine[1] || theirs[1] != mine[0]))
            st = fail_to(e, PG_ERR_COMM,
                         "party %d sent %llu bytes to party %d, which received %llu; party %d sent %llu bytes "
                         "to party %d, which received %llu",
                         i, (unsigned long long)theirs[0], p->party, (unsigned long long)mine[1], p->party,
                         (unsigned long long)mine[0], i, (unsigned long long)theirs[1]);
        if (st && !first) {
            first = st;
            first_err = e;
        }
    }
    // nothing may be left unread of the step's messages (a duplicate)
    for (int i = 0; i < p->n && !first; i++) {
        if (i == p->party) continue;
        pollfd pf = {p->rcv[i][0], POLLIN, 0};
        if (poll(&pf, 1, 20) > 0 && (pf.revents & POLLIN)) {
            uint8_t byte;
            if (recv(p->rcv[i][0], &byte, 1, MSG_PEEK | MSG_DONTWAIT) > 0) {
                first = PG_ERR_COMM;
                fail_to(first_err, PG_ERR_COMM, "unexpected bytes from party %d after its last message", i);
            }
        }
    }
    if (first) return p->fail(first, "%s", first_err.c_str());
    return PG_OK;
}

}  // extern "C"

// ---------------------------------------------------- device messages and steps

namespace {

int grow_pinned(pg_party *p, void *&buf, size_t &have, size_t bytes) {
    if (bytes <= have) return PG_OK;
    if (buf) cudaFreeHost(buf);
    buf = nullptr;
    have = 0;
    if (cudaMallocHost(&buf, bytes) != cudaSuccess) {
        cudaGetLastError();
        buf = nullptr;
        return p->fail(PG_ERR_NO_MEMORY, "pinned staging of %zu bytes", bytes);
    }
    have = bytes;
    return PG_OK;
}

// transmit (to, dev_out) while receiving (from, dev_in): the send runs on its
// own thread, as the reference's DeviceData::transmit does
int exchange(pg_party *p, Ctx *c, int to, const void *dev_out, size_t bytes_out, int from, void *dev_in,
             size_t bytes_in) {
    int st = PG_OK;
    if (to >= 0 && (st = grow_pinned(p, p->stage_out, p->stage_out_bytes, bytes_out))) return st;
    if (from >= 0 && (st = grow_pinned(p, p->stage_in, p->stage_in_bytes, bytes_in))) return st;
    if (to >= 0 && bytes_out) {
        PG_CHECK_CUDA(c, cudaMemcpyAsync(p->stage_out, dev_out, bytes_out, cudaMemcpyDeviceToHost, c->stream));
        PG_CHECK_CUDA(c, cudaStreamSynchronize(c->stream));
    }
    int st_send = PG_OK;
    std::string send_err, recv_err;
    std::thread sender;
    if (to >= 0) sender = std::thread([&] { st_send = party_send(p, to, p->stage_out, bytes_out, send_err); });
    if (from >= 0) st = party_recv(p, from, p->stage_in, bytes_in, recv_err);
    if (sender.joinable()) sender.join();
    if (st_send) return p->fail(st_send, "%s", send_err.c_str());
    if (st) return p->fail(st, "%s", recv_err.c_str());
    if (from >= 0 && bytes_in) {
        PG_CHECK_CUDA(c, cudaMemcpyAsync(dev_in, p->stage_in, bytes_in, cudaMemcpyHostToDevice, c->stream));
        PG_CHECK_CUDA(c, cudaStreamSynchronize(c->stream));
    }
    return PG_OK;
}

__global__ void add3_kernel(const uint64_t *a, const uint64_t *b, const uint64_t *d, uint64_t *out, size_t n) {
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
        out[i] = a[i] + b[i] + d[i];
}

// z = a x b accumulated: c += acc (localMatMul's c += acc)
__global__ void accumulate_kernel(uint64_t *c, const uint64_t *acc, size_t n) {
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
        c[i] += acc[i];
}

// dividePublic3out3's end at one party: q = (z + r1 + r2) / d through double;
// out = r + q with r = 1 and q at party A's shareA and party C's shareB
__global__ void divide3_kernel(const uint64_t *z, const uint64_t *r1, const uint64_t *r2, uint64_t d, int dshift,
                               int party, uint64_t *out0, uint64_t *out1, size_t n) {
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
        const uint64_t v = 1 + div_public<uint64_t>(z[i] + r1[i] + r2[i], d, dshift);
        out0[i] = party == 0 ? v : 0;
        out1[i] = party == 2 ? v : 0;
    }
}

__global__ void sub_scalar_kernel(uint64_t *a, uint64_t v, size_t n) {
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
        a[i] -= v;
}

unsigned blocks_for(Ctx *c, size_t n) {
    const size_t b = (n + 255) / 256;
    const size_t cap = (size_t)(c->sm_count > 0 ? c->sm_count : 148) * 8;
    return (unsigned)(b < 1 ? 1 : b > cap ? cap : b);
}

}  // namespace

// the context's error text becomes the party's when a GPU call fails
template <typename F> static int party_step(pg_party *p, pg_ctx *c, F f) {
    if (!p) return PG_ERR_INVALID_ARG;
    p->err.clear();
    const int st = f();
    if (st && p->err.empty() && c) p->err = c->err;
    return st;
}

extern "C" {

static int pg_party_exchange_impl(pg_party *p, pg_ctx *ctx, int to, const void *dev_out, size_t bytes_out, int from,
                      void *dev_in, size_t bytes_in) {
    if (!p || !ctx) return PG_ERR_INVALID_ARG;
    return exchange(p, ctx, to, dev_out, bytes_out, from, dev_in, bytes_in);
}

static int pg_party_rss_reconstruct_u64_impl(pg_party *p, pg_ctx *c, const uint64_t *const sh[2], size_t n, uint64_t *out) {
    if (!p || !c || !sh || !out || (n && (!sh[0] || !sh[1]))) return PG_ERR_INVALID_ARG;
    if (p->n != 3) return p->fail(PG_ERR_UNSUPPORTED, "RSS needs 3 parties, not %d", p->n);
    const int next = (p->party + 1) % 3, prev = (p->party + 2) % 3;
    uint64_t *rx = (uint64_t *)scratch(c, n * 8 + 8);
    if (!rx) return PG_ERR_NO_MEMORY;
    int st = exchange(p, c, next, sh[0], n * 8, prev, rx, n * 8);
    if (st) return st;
    if (n) {
        add3_kernel<<<blocks_for(c, n), 256, 0, c->stream>>>(sh[0], sh[1], rx, out, n);
        c->launches++;
        if ((st = launch_status(c, "add3_kernel"))) return st;
    }
    p->rounds++;
    return PG_OK;
}

static int pg_party_rss_reshare_u64_impl(pg_party *p, pg_ctx *c, const uint64_t *cin, size_t n, uint64_t *const out[2]) {
    if (!p || !c || !out || (n && (!cin || !out[0] || !out[1]))) return PG_ERR_INVALID_ARG;
    if (p->n != 3) return p->fail(PG_ERR_UNSUPPORTED, "RSS needs 3 parties, not %d", p->n);
    const int next = (p->party + 1) % 3, prev = (p->party + 2) % 3;
    if (n) PG_CHECK_CUDA(c, cudaMemcpyAsync(out[0], cin, n * 8, cudaMemcpyDeviceToDevice, c->stream));
    int st = exchange(p, c, prev, out[0], n * 8, next, out[1], n * 8);
    if (st) return st;
    p->rounds++;
    return PG_OK;
}

static int pg_party_rss_matmul_u64_impl(pg_party *p, pg_ctx *c, const uint64_t *const a[2], const uint64_t *const b[2],
                            uint64_t *const out[2], int M, int N, int K, int tA, int tB, int tC, int trunc) {
    if (!p || !c || !a || !b || !out || !a[0] || !a[1] || !b[0] || !b[1] || !out[0] || !out[1])
        return PG_ERR_INVALID_ARG;
    if (p->n != 3) return p->fail(PG_ERR_UNSUPPORTED, "RSS needs 3 parties, not %d", p->n);
    if (M <= 0 || N <= 0 || K <= 0 || trunc < 0 || trunc > 62) return set_error(c, PG_ERR_SIZE, "party matmul sizes");
    const size_t mn = (size_t)M * N;
    const int next = (p->party + 1) % 3, prev = (p->party + 2) % 3;
    uint64_t *z = (uint64_t *)scratch(c, 4 * mn * 8);
    if (!z) return PG_ERR_NO_MEMORY;
    uint64_t *acc = z + mn, *r1 = z + 2 * mn, *r2 = z + 3 * mn;
    // localMatMul (RSS.inl:1096-1110): z = a0 b0 + a0 b1 + a1 b0
    PG_CHECK_CUDA(c, cudaMemsetAsync(z, 0, mn * 8, c->stream));
    const uint64_t *pairs[3][2] = {{a[0], b[0]}, {a[0], b[1]}, {a[1], b[0]}};
    int st = PG_OK;
    for (int t = 0; t < 3 && !st; t++) {
        st = plain_gemm<uint64_t>(c, M, N, K, pairs[t][0], tA, pairs[t][1], tB, acc, tC);
        if (!st) {
            accumulate_kernel<<<blocks_for(c, mn), 256, 0, c->stream>>>(z, acc, mn);
            c->launches++;
            st = launch_status(c, "accumulate_kernel");
        }
    }
    if (st) return st;
    // dividePublic3out3 (RSS.inl:1076-1094): r' = d held by party A only
    const uint64_t d = 1ull << trunc;
    if (p->party == 0) {
        sub_scalar_kernel<<<blocks_for(c, mn), 256, 0, c->stream>>>(z, d, mn);
        c->launches++;
        if ((st = launch_status(c, "sub_scalar_kernel"))) return st;
    }
    // reconstruct3out3 (RSS.inl:1019-1050): to next / from previous, then to previous / from next
    if ((st = exchange(p, c, next, z, mn * 8, prev, r1, mn * 8))) return st;
    if ((st = exchange(p, c, prev, z, mn * 8, next, r2, mn * 8))) return st;
    divide3_kernel<<<blocks_for(c, mn), 256, 0, c->stream>>>(z, r1, r2, d, pow2_shift<uint64_t>(d), p->party, out[0],
                                                            out[1], mn);
    c->launches++;
    if ((st = launch_status(c, "divide3_kernel"))) return st;
    p->rounds++;
    return PG_OK;
}



int pg_party_exchange(pg_party *p, pg_ctx *ctx, int to, const void *dev_out, size_t bytes_out, int from,
                      void *dev_in, size_t bytes_in) {
    return party_step(p, ctx, [&] { return pg_party_exchange_impl(p, ctx, to, dev_out, bytes_out, from, dev_in, bytes_in); });
}
int pg_party_rss_reconstruct_u64(pg_party *p, pg_ctx *c, const uint64_t *const sh[2], size_t n, uint64_t *out) {
    return party_step(p, c, [&] { return pg_party_rss_reconstruct_u64_impl(p, c, sh, n, out); });
}
int pg_party_rss_reshare_u64(pg_party *p, pg_ctx *c, const uint64_t *cin, size_t n, uint64_t *const out[2]) {
    return party_step(p, c, [&] { return pg_party_rss_reshare_u64_impl(p, c, cin, n, out); });
}
int pg_party_rss_matmul_u64(pg_party *p, pg_ctx *c, const uint64_t *const a[2], const uint64_t *const b[2],
                            uint64_t *const out[2], int M, int N, int K, int tA, int tB, int tC, int trunc) {
    return party_step(p, c, [&] { return pg_party_rss_matmul_u64_impl(p, c, a, b, out, M, N, K, tA, tB, tC, trunc); });
}

}  // extern "C"
