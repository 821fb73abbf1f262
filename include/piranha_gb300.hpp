/*
 * piranha_gb300.hpp — the reference's C++ share-class surface on top of the C
 * ABI of piranha_gb300.h, for a Piranha build that runs its three parties
 * simulated on one GPU.
 *
 * It keeps the names, argument order and meaning of Piranha's hot-path API so
 * that code written against it compiles unchanged in simulation mode:
 *   - DeviceData<T>            src/gpu/DeviceData.h:51-277 (owning device array
 *                              and its elementwise operators, functors.cuh)
 *   - RSS<T>                   src/mpc/RSS.h:15-101 (here: all three parties'
 *                              share pairs, six device buffers [party*2+share])
 *   - dividePublic, reconstruct, matmul, selectShare, convolution, dReLU,
 *     ReLU, maxpool, reshare   src/mpc/RSS.h:105-145
 *   - gpu::gemm                src/gpu/gemm.cuh:102-112
 *   - gpu::conv_fprop / conv_dgrad / conv_wgrad   src/gpu/conv.cuh:379-490
 *   - gpu::maxpool_im2row, gpu::truncate_cols, gpu::elementVectorAdd,
 *     gpu::reduceSum           src/gpu/convolution.cuh:252-304, matrix.cuh
 *   - cutlass::conv::Operator  (redefined here: CUTLASS is not a dependency)
 *
 * Differences a caller sees, all due to the simulation:
 *   - an RSS<T> holds every party's shares, so getShare(i) names share i of
 *     all three parties at once, and reconstruct(in, out) writes party A's
 *     reveal (reconstruct(in, out[3]) writes each party's);
 *   - errors throw piranha_gb300::Error (the status and pg_last_error's text)
 *     where Piranha asserts or exits;
 *   - calls are ordered on the context's stream and do not synchronize;
 *     download() and piranha_gb300::sync() do.
 * Every computation runs in the library's CUDA kernels; nothing here computes
 * on the host except fixed-point encoding of host values. Link with
 * -lpiranha_gb300 -lcudart.
 */
#ifndef PIRANHA_GB300_HPP
#define PIRANHA_GB300_HPP

#include <cuda_runtime.h>

#include <cmath>
#include <cstdint>
#include <initializer_list>
#include <stdexcept>
#include <string>
#include <type_traits>
#include <utility>
#include <vector>

#include "piranha_gb300.h"

#ifndef FLOAT_PRECISION
#define FLOAT_PRECISION 26 /* src/globals.h:19-21 */
#endif

namespace piranha_gb300 {

class Error : public std::runtime_error {
  public:
    Error(int st, const std::string &msg) : std::runtime_error(msg), status(st) {}
    int status;
};

/* The one context that stands in for the reference's process globals
 * (partyNum, PrecomputeObject, comm_profiler): created on device 0 at first
 * use, or set by the caller (who keeps ownership). */
inline pg_ctx *&context_slot() {
    static pg_ctx *ctx = nullptr;
    return ctx;
}
inline pg_ctx *context() {
    pg_ctx *&c = context_slot();
    if (!c) {
        const int st = pg_ctx_create(&c, 0);
        if (st != PG_OK) {
            c = nullptr;
            throw Error(st, "pg_ctx_create(device 0) failed");
        }
    }
    return c;
}
inline void set_context(pg_ctx *ctx) { context_slot() = ctx; }
inline void check(int st) {
    if (st != PG_OK) throw Error(st, pg_last_error(context()));
}
inline void check_cuda(cudaError_t e, const char *what) {
    if (e != cudaSuccess) throw Error(PG_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
}
inline cudaStream_t stream() { return (cudaStream_t)pg_ctx_get_stream(context()); }
inline void sync() { check(pg_sync(context())); }

/* (T)(f * 2^FLOAT_PRECISION) as the reference's x86-64 hosts computed it: the
 * double is truncated toward zero into a signed integer first
 * (src/util/util.cuh:28-33, src/mpc/RSS.inl:126,397). */
template <typename T> inline T encode(double v, bool fixed = true) {
    const double x = fixed ? v * (double)(1ull << FLOAT_PRECISION) : v;
    return (T)(uint64_t)(int64_t)x;
}

}  // namespace piranha_gb300

/* ------------------------------------------------------------- DeviceData */

template <typename T> class DeviceData {
    static_assert(std::is_same<T, uint64_t>::value || std::is_same<T, uint32_t>::value ||
                      std::is_same<T, uint8_t>::value,
                  "DeviceData<T>: T is uint64_t, uint32_t or uint8_t");

  public:
    explicit DeviceData(size_t n = 0) { resize(n); }
    DeviceData(std::initializer_list<T> vals) {
        resize(vals.size());
        upload(std::vector<T>(vals));
    }
    DeviceData(const DeviceData &) = delete;
    DeviceData &operator=(const DeviceData &) = delete;
    DeviceData(DeviceData &&o) noexcept : ptr_(o.ptr_), n_(o.n_) {
        o.ptr_ = nullptr;
        o.n_ = 0;
    }
    ~DeviceData() { release(); }

    size_t size() const { return n_; }
    T *data() { return ptr_; }
    const T *data() const { return ptr_; }

    /* a new size; the contents are zero afterwards */
    void resize(size_t n) {
        if (n != n_ || !ptr_) {
            release();
            piranha_gb300::check_cuda(cudaMalloc((void **)&ptr_, (n ? n : 1) * sizeof(T)), "cudaMalloc");
            n_ = n;
        }
        zero();
    }
    void zero() {
        if (n_) piranha_gb300::check_cuda(cudaMemsetAsync(ptr_, 0, n_ * sizeof(T), piranha_gb300::stream()), "memset");
    }
    void fill(T v) {
        if (std::is_same<T, uint64_t>::value)
            piranha_gb300::check(pg_device_op_u64(piranha_gb300::context(), PG_OP_SET, (uint64_t *)ptr_, n_,
                                                  PG_RHS_SCALAR, (uint64_t)v, nullptr));
        else if (std::is_same<T, uint8_t>::value)
            piranha_gb300::check_cuda(cudaMemsetAsync(ptr_, (int)v, n_, piranha_gb300::stream()), "memset");
        else
            throw piranha_gb300::Error(PG_ERR_UNSUPPORTED, "DeviceData<uint32_t>::fill");
    }
    void upload(const std::vector<T> &h) {
        if (h.size() != n_) throw piranha_gb300::Error(PG_ERR_SIZE, "DeviceData::upload: size");
        if (n_)
            piranha_gb300::check_cuda(cudaMemcpyAsync(ptr_, h.data(), n_ * sizeof(T), cudaMemcpyHostToDevice,
                                                      piranha_gb300::stream()),
                                      "upload");
        piranha_gb300::sync();
    }
    std::vector<T> download() const {
        std::vector<T> h(n_);
        piranha_gb300::sync();
        if (n_) piranha_gb300::check_cuda(cudaMemcpy(h.data(), ptr_, n_ * sizeof(T), cudaMemcpyDeviceToHost), "download");
        return h;
    }

    /* the elementwise operators of DeviceData (functors.cuh), uint64_t */
#define PG_DD_OP(sym, code)                                                                                       \
    DeviceData &operator sym(T rhs) { return apply(code, PG_RHS_SCALAR, rhs, nullptr); }                          \
    DeviceData &operator sym(const DeviceData &rhs) {                                                             \
        if (rhs.size() != n_) throw piranha_gb300::Error(PG_ERR_SIZE, "DeviceData operator: sizes differ");      \
        return apply(code, PG_RHS_PUBLIC, 0, rhs.data());                                                         \
    }
    PG_DD_OP(+=, PG_OP_ADD)
    PG_DD_OP(-=, PG_OP_SUB)
    PG_DD_OP(*=, PG_OP_MUL)
    PG_DD_OP(/=, PG_OP_DIV)
    PG_DD_OP(^=, PG_OP_XOR)
    PG_DD_OP(&=, PG_OP_AND)
    PG_DD_OP(>>=, PG_OP_SHR)
    PG_DD_OP(<<=, PG_OP_SHL)
#undef PG_DD_OP

  private:
    DeviceData &apply(int op, int kind, T scalar, const T *vec) {
        if (!std::is_same<T, uint64_t>::value)
            throw piranha_gb300::Error(PG_ERR_UNSUPPORTED, "DeviceData operators are built for uint64_t");
        piranha_gb300::check(pg_device_op_u64(piranha_gb300::context(), op, (uint64_t *)ptr_, n_, kind,
                                              (uint64_t)scalar, (const uint64_t *)vec));
        return *this;
    }
    void release() {
        if (ptr_) {
            cudaStreamSynchronize(piranha_gb300::stream());
            cudaFree(ptr_);
        }
        ptr_ = nullptr;
        n_ = 0;
    }
    T *ptr_ = nullptr;
    size_t n_ = 0;
};

/* -------------------------------------------------------------------- RSS */

template <typename T> class RSS;

/* Share i of every party (RSSBase::getShare, RSS.inl:144-168, in simulation):
 * adding a public vector to it adds it to all three parties' share i. */
template <typename T> class SharePart {
  public:
    SharePart(RSS<T> *owner, int i) : owner_(owner), i_(i) {}
    size_t size() const;
    T *party(int p) const;
    RSS<T> &owner() const { return *owner_; }
    int index() const { return i_; }
    SharePart &operator+=(const DeviceData<T> &v) { return apply(PG_OP_ADD, v); }
    SharePart &operator-=(const DeviceData<T> &v) { return apply(PG_OP_SUB, v); }
    SharePart *operator->() { return this; }
    SharePart &operator*() { return *this; }

  private:
    SharePart &apply(int op, const DeviceData<T> &v);
    RSS<T> *owner_;
    int i_;
};

template <typename T> class RSS {
  public:
    typedef T share_type;
    static const int numParties = 3;
    static int numShares() { return 2; }

    explicit RSS(size_t n) { alloc(n); }
    /* RSS(std::initializer_list<double>, bool) (RSS.inl:389-414): party A's
     * shareA and party C's shareB hold the values */
    RSS(std::initializer_list<double> vals, bool convertToFixedPoint = true) {
        alloc(vals.size());
        std::vector<T> x;
        for (double v : vals) x.push_back(piranha_gb300::encode<T>(v, convertToFixedPoint));
        upload(0, 0, x);
        upload(2, 1, x);
    }
    RSS(const RSS &) = delete;
    RSS &operator=(const RSS &) = delete;
    RSS(RSS &&o) noexcept : n_(o.n_) {
        for (int k = 0; k < 6; k++) {
            buf_[k] = o.buf_[k];
            o.buf_[k] = nullptr;
        }
        o.n_ = 0;
    }
    ~RSS() { release(); }

    size_t size() const { return n_; }
    /* a new size; every share is zero afterwards */
    void resize(size_t n) {
        if (n == n_) return;
        release();
        alloc(n);
    }
    void zero() {
        for (int k = 0; k < 6; k++)
            if (n_) piranha_gb300::check_cuda(cudaMemsetAsync(buf_[k], 0, n_ * sizeof(T), piranha_gb300::stream()), "memset");
    }
    /* RSSBase::fill (RSS.inl:117-121): party A's shareA and party C's shareB
     * hold val, the other shares 0 */
    void fill(T val) {
        zero();
        fill_buffer(0, val);
        fill_buffer(5, val);
    }
    /* RSSBase::setPublic (RSS.inl:123-142), with the fall-through of its
     * PARTY_B case: party B's shareB holds the values too */
    void setPublic(const std::vector<double> &v) {
        if (v.size() != n_) throw piranha_gb300::Error(PG_ERR_SIZE, "setPublic: size");
        std::vector<T> x;
        for (double f : v) x.push_back(piranha_gb300::encode<T>(f));
        zero();
        upload(0, 0, x);
        upload(1, 1, x);
        upload(2, 1, x);
    }

    SharePart<T> getShare(int i) {
        if (i < 0 || i > 1) throw piranha_gb300::Error(PG_ERR_INVALID_ARG, "getShare: index");
        return SharePart<T>(this, i);
    }
    T *buffer(int party, int share) const { return buf_[party * 2 + share]; }
    T *const *buffers() { return buf_; }
    const T *const *buffers() const { return (const T *const *)buf_; }

    /* one party's share, copied to the host (synchronizes) */
    std::vector<T> download(int party, int share) const {
        std::vector<T> h(n_);
        piranha_gb300::sync();
        if (n_)
            piranha_gb300::check_cuda(cudaMemcpy(h.data(), buffer(party, share), n_ * sizeof(T), cudaMemcpyDeviceToHost),
                                      "download");
        return h;
    }
    void upload(int party, int share, const std::vector<T> &h) {
        if (h.size() != n_) throw piranha_gb300::Error(PG_ERR_SIZE, "RSS::upload: size");
        if (n_)
            piranha_gb300::check_cuda(cudaMemcpyAsync(buffer(party, share), h.data(), n_ * sizeof(T),
                                                      cudaMemcpyHostToDevice, piranha_gb300::stream()),
                                      "upload");
        piranha_gb300::sync();
    }

    /* local operators (RSS.inl:168-345) */
    RSS &operator+=(T rhs) { return local(PG_OP_ADD, PG_RHS_SCALAR, rhs, nullptr, nullptr); }
    RSS &operator-=(T rhs) { return local(PG_OP_SUB, PG_RHS_SCALAR, rhs, nullptr, nullptr); }
    RSS &operator*=(T rhs) { return local(PG_OP_MUL, PG_RHS_SCALAR, rhs, nullptr, nullptr); }
    RSS &operator>>=(T rhs) { return local(PG_OP_SHR, PG_RHS_SCALAR, rhs, nullptr, nullptr); }
#define PG_RSS_PUB(sym, code)                                                                                \
    RSS &operator sym(const DeviceData<T> &rhs) {                                                          \
        if (rhs.size() != n_) throw piranha_gb300::Error(PG_ERR_SIZE, "RSS operator: sizes differ");       \
        return local(code, PG_RHS_PUBLIC, 0, rhs.data(), nullptr);                                         \
    }
    PG_RSS_PUB(+=, PG_OP_ADD)
    PG_RSS_PUB(-=, PG_OP_SUB)
    PG_RSS_PUB(*=, PG_OP_MUL)
    PG_RSS_PUB(^=, PG_OP_XOR)
    PG_RSS_PUB(&=, PG_OP_AND)
    PG_RSS_PUB(>>=, PG_OP_SHR)
    PG_RSS_PUB(<<=, PG_OP_SHL)
#undef PG_RSS_PUB
    RSS &operator+=(const RSS &rhs) { return local(PG_OP_ADD, PG_RHS_SHARES, 0, nullptr, &rhs); }
    RSS &operator-=(const RSS &rhs) { return local(PG_OP_SUB, PG_RHS_SHARES, 0, nullptr, &rhs); }
    RSS &operator^=(const RSS &rhs) { return local(PG_OP_XOR, PG_RHS_SHARES, 0, nullptr, &rhs); }
    /* the protocol steps RSS *= RSS and &= RSS (RSS.inl:283-345): one round */
    RSS &operator*=(const RSS &rhs) {
        same_size(rhs);
        piranha_gb300::check(pg_rss_mul_u64(piranha_gb300::context(), (uint64_t *const *)buf_,
                                            (const uint64_t *const *)rhs.buf_, n_));
        return *this;
    }
    RSS &operator&=(const RSS &rhs) {
        same_size(rhs);
        if (std::is_same<T, uint8_t>::value)
            piranha_gb300::check(pg_rss_and_u8(piranha_gb300::context(), (uint8_t *const *)buf_,
                                               (const uint8_t *const *)rhs.buf_, n_));
        else
            piranha_gb300::check(pg_rss_and_u64(piranha_gb300::context(), (uint64_t *const *)buf_,
                                                (const uint64_t *const *)rhs.buf_, n_));
        return *this;
    }

    void same_size(const RSS &o) const {
        if (o.n_ != n_) throw piranha_gb300::Error(PG_ERR_SIZE, "RSS: sizes differ");
    }

  private:
    RSS &local(int op, int kind, T scalar, const T *pub, const RSS *sh) {
        if (!std::is_same<T, uint64_t>::value)
            throw piranha_gb300::Error(PG_ERR_UNSUPPORTED, "RSS local operators are built for uint64_t");
        if (sh) same_size(*sh);
        piranha_gb300::check(pg_rss_local_u64(piranha_gb300::context(), op, (uint64_t *const *)buf_, n_, kind,
                                              (uint64_t)scalar, (const uint64_t *)pub,
                                              sh ? (const uint64_t *const *)sh->buf_ : nullptr));
        return *this;
    }
    void fill_buffer(int k, T val) {
        if (!n_) return;
        if (std::is_same<T, uint64_t>::value)
            piranha_gb300::check(pg_device_op_u64(piranha_gb300::context(), PG_OP_SET, (uint64_t *)buf_[k], n_,
                                                  PG_RHS_SCALAR, (uint64_t)val, nullptr));
        else if (std::is_same<T, uint8_t>::value)
            piranha_gb300::check_cuda(cudaMemsetAsync(buf_[k], (int)val, n_, piranha_gb300::stream()), "memset");
        else
            throw piranha_gb300::Error(PG_ERR_UNSUPPORTED, "RSS<uint32_t>::fill");
    }
    void alloc(size_t n) {
        void *p[6];
        piranha_gb300::check(pg_alloc_shares(piranha_gb300::context(), 6, n, (int)sizeof(T), p));
        for (int k = 0; k < 6; k++) buf_[k] = (T *)p[k];
        n_ = n;
    }
    void release() {
        if (buf_[0]) pg_free_shares(piranha_gb300::context(), buf_[0]);
        for (int k = 0; k < 6; k++) buf_[k] = nullptr;
        n_ = 0;
    }
    T *buf_[6] = {nullptr, nullptr, nullptr, nullptr, nullptr, nullptr};
    size_t n_ = 0;
};

template <typename T> size_t SharePart<T>::size() const { return owner_->size(); }
template <typename T> T *SharePart<T>::party(int p) const { return owner_->buffer(p, i_); }
template <typename T> SharePart<T> &SharePart<T>::apply(int op, const DeviceData<T> &v) {
    static_assert(std::is_same<T, uint64_t>::value, "share additions are built for uint64_t");
    if (v.size() != size()) throw piranha_gb300::Error(PG_ERR_SIZE, "share operator: sizes differ");
    for (int p = 0; p < 3; p++)
        piranha_gb300::check(pg_device_op_u64(piranha_gb300::context(), op, (uint64_t *)party(p), size(),
                                              PG_RHS_PUBLIC, 0, (const uint64_t *)v.data()));
    return *this;
}

/* ------------------------------------------------- protocol free functions */

namespace cutlass {
namespace conv {
enum class Operator { kFprop = PG_CONV_FPROP, kDgrad = PG_CONV_DGRAD, kWgrad = PG_CONV_WGRAD };
}  // namespace conv
}  // namespace cutlass

/* dividePublic(RSS&, T) (RSS.inl:423-440) */
inline void dividePublic(RSS<uint64_t> &a, uint64_t denominator) {
    piranha_gb300::check(pg_rss_divide_public_u64(piranha_gb300::context(), a.buffers(), a.size(), denominator));
}
inline void dividePublic(RSS<uint32_t> &a, uint32_t denominator) {
    piranha_gb300::check(pg_rss_divide_public_u32(piranha_gb300::context(), a.buffers(), a.size(), denominator));
}
/* dividePublic(RSS&, DeviceData&) (RSS.inl:442-455) */
inline void dividePublic(RSS<uint64_t> &a, DeviceData<uint64_t> &denominators) {
    if (denominators.size() != a.size()) throw piranha_gb300::Error(PG_ERR_SIZE, "dividePublic: sizes differ");
    piranha_gb300::check(
        pg_rss_divide_public_vec_u64(piranha_gb300::context(), a.buffers(), a.size(), denominators.data()));
}

/* reconstruct (RSS.inl:457-479): every party's reveal, or party A's */
inline void reconstruct(const RSS<uint64_t> &in, DeviceData<uint64_t> (&out)[3]) {
    uint64_t *o[3];
    for (int p = 0; p < 3; p++) {
        if (out[p].size() != in.size()) out[p].resize(in.size());
        o[p] = out[p].data();
    }
    piranha_gb300::check(pg_rss_reconstruct_u64(piranha_gb300::context(), in.buffers(), in.size(), o));
}
inline void reconstruct(const RSS<uint8_t> &in, DeviceData<uint8_t> (&out)[3]) {
    uint8_t *o[3];
    for (int p = 0; p < 3; p++) {
        if (out[p].size() != in.size()) out[p].resize(in.size());
        o[p] = out[p].data();
    }
    piranha_gb300::check(pg_rss_reconstruct_u8(piranha_gb300::context(), in.buffers(), in.size(), o));
}
template <typename T> inline void reconstruct(const RSS<T> &in, DeviceData<T> &out) {
    DeviceData<T> all[3];
    reconstruct(in, all);
    if (out.size() != in.size()) out.resize(in.size());
    if (in.size())
        piranha_gb300::check_cuda(cudaMemcpyAsync(out.data(), all[0].data(), in.size() * sizeof(T),
                                                  cudaMemcpyDeviceToDevice, piranha_gb300::stream()),
                                  "reconstruct");
}

/* reshare (RSS.inl:1052-1074): c[p] is party p's 3-out-of-3 share */
inline void reshare(DeviceData<uint64_t> (&c)[3], RSS<uint64_t> &out) {
    const uint64_t *cin[3] = {c[0].data(), c[1].data(), c[2].data()};
    piranha_gb300::check(pg_rss_reshare_u64(piranha_gb300::context(), cin, out.size(), out.buffers()));
}

/* matmul (RSS.inl:481-540): c = (a x b) / 2^truncation, layouts as gpu::gemm */
inline void matmul(const RSS<uint64_t> &a, const RSS<uint64_t> &b, RSS<uint64_t> &c, int M, int N, int K,
                   bool transpose_a, bool transpose_b, bool transpose_c, uint64_t truncation) {
    piranha_gb300::check(pg_rss_matmul_u64(piranha_gb300::context(), a.buffers(), b.buffers(), c.buffers(), M, N, K,
                                           transpose_a, transpose_b, transpose_c, (int)truncation));
}
inline void matmul(const RSS<uint32_t> &a, const RSS<uint32_t> &b, RSS<uint32_t> &c, int M, int N, int K,
                   bool transpose_a, bool transpose_b, bool transpose_c, uint32_t truncation) {
    piranha_gb300::check(pg_rss_matmul_u32(piranha_gb300::context(), a.buffers(), b.buffers(), c.buffers(), M, N, K,
                                           transpose_a, transpose_b, transpose_c, (int)truncation));
}

/* selectShare (RSS.inl:542-569): z = b ? y : x */
inline void selectShare(const RSS<uint64_t> &x, const RSS<uint64_t> &y, const RSS<uint8_t> &b, RSS<uint64_t> &z) {
    piranha_gb300::check(pg_rss_select_share_u64_u8(piranha_gb300::context(), x.buffers(), y.buffers(), b.buffers(),
                                                    z.buffers(), x.size()));
}
inline void selectShare(const RSS<uint64_t> &x, const RSS<uint64_t> &y, const RSS<uint64_t> &b, RSS<uint64_t> &z) {
    piranha_gb300::check(pg_rss_select_share_u64_u64(piranha_gb300::context(), x.buffers(), y.buffers(), b.buffers(),
                                                     z.buffers(), x.size()));
}

/* convolution (RSS.inl:706-803) */
inline void convolution(const RSS<uint64_t> &A, const RSS<uint64_t> &B, RSS<uint64_t> &C, cutlass::conv::Operator op,
                        int batchSize, int imageHeight, int imageWidth, int filterSize, int Din, int Dout,
                        int stride, int padding, int truncation) {
    piranha_gb300::check(pg_rss_conv_u64(piranha_gb300::context(), A.buffers(), B.buffers(), C.buffers(), (int)op,
                                         batchSize, imageHeight, imageWidth, filterSize, Din, Dout, stride, padding,
                                         truncation));
}

/* dReLU (RSS.inl:806-852) */
inline void dReLU(const RSS<uint64_t> &in, RSS<uint8_t> &result) {
    piranha_gb300::check(pg_rss_drelu_u64_u8(piranha_gb300::context(), in.buffers(), in.size(), result.buffers()));
}
inline void dReLU(const RSS<uint64_t> &in, RSS<uint64_t> &result) {
    piranha_gb300::check(pg_rss_drelu_u64_u64(piranha_gb300::context(), in.buffers(), in.size(), result.buffers()));
}

/* ReLU (RSS.inl:854-865) */
inline void ReLU(const RSS<uint64_t> &in, RSS<uint64_t> &result, RSS<uint8_t> &dresult) {
    piranha_gb300::check(pg_rss_relu_u64_u8(piranha_gb300::context(), in.buffers(), in.size(), result.buffers(),
                                            dresult.buffers()));
}
inline void ReLU(const RSS<uint64_t> &in, RSS<uint64_t> &result, RSS<uint64_t> &dresult) {
    piranha_gb300::check(pg_rss_relu_u64_u64(piranha_gb300::context(), in.buffers(), in.size(), result.buffers(),
                                             dresult.buffers()));
}
inline void ReLU(const RSS<uint32_t> &in, RSS<uint32_t> &result, RSS<uint8_t> &dresult) {
    piranha_gb300::check(pg_rss_relu_u32_u8(piranha_gb300::context(), in.buffers(), in.size(), result.buffers(),
                                            dresult.buffers()));
}

/* maxpool (RSS.inl:867-1017) over rows of k values */
inline void maxpool(const RSS<uint64_t> &in, RSS<uint64_t> &result, RSS<uint8_t> &dresult, int k) {
    piranha_gb300::check(pg_rss_maxpool_u64_u8(piranha_gb300::context(), in.buffers(), in.size(), k, result.buffers(),
                                               dresult.buffers()));
}
inline void maxpool(const RSS<uint64_t> &in, RSS<uint64_t> &result, RSS<uint64_t> &dresult, int k) {
    piranha_gb300::check(pg_rss_maxpool_u64_u64(piranha_gb300::context(), in.buffers(), in.size(), k,
                                                result.buffers(), dresult.buffers()));
}

/* ------------------------------------------------------------ gpu kernels */

namespace gpu {

/* gpu::gemm (gemm.cuh:102-112): C = A x B mod 2^w; an operand is row-major
 * when its transpose flag is set, column-major otherwise */
inline void gemm(int M, int N, int K, const DeviceData<uint64_t> *A, bool transpose_a, const DeviceData<uint64_t> *B,
                 bool transpose_b, DeviceData<uint64_t> *C, bool transpose_c) {
    piranha_gb300::check(pg_gemm_u64(piranha_gb300::context(), M, N, K, A->data(), transpose_a, B->data(), transpose_b,
                                      C->data(), transpose_c));
}
inline void gemm(int M, int N, int K, const DeviceData<uint32_t> *A, bool transpose_a, const DeviceData<uint32_t> *B,
                 bool transpose_b, DeviceData<uint32_t> *C, bool transpose_c) {
    piranha_gb300::check(pg_gemm_u32(piranha_gb300::context(), M, N, K, A->data(), transpose_a, B->data(), transpose_b,
                                      C->data(), transpose_c));
}

/* conv_fprop (conv.cuh:379-403): A = X (b, H, W, Din), B = F (Dout, fh, fw,
 * Din), C = Y; square filters, equal paddings, dilation 1 */
inline void conv_fprop(const DeviceData<uint64_t> *A, const DeviceData<uint64_t> *B, DeviceData<uint64_t> *C, int b,
                       int imageHeight, int imageWidth, int Din, int Dout, int filterHeight, int filterWidth,
                       int paddingHeight, int paddingWidth, int stride, int dilation) {
    if (filterHeight != filterWidth || paddingHeight != paddingWidth || dilation != 1)
        throw piranha_gb300::Error(PG_ERR_UNSUPPORTED, "conv_fprop: square filters, equal paddings, dilation 1");
    piranha_gb300::check(pg_conv_u64(piranha_gb300::context(), PG_CONV_FPROP, b, imageHeight, imageWidth, Din, Dout,
                                      filterHeight, filterWidth, paddingHeight, stride, A->data(), B->data(),
                                      C->data()));
}
/* conv_dgrad (conv.cuh:425-447): A = dY (b, dh, dw, Dout), B = F, C = dX (b, H, W, Din) */
inline void conv_dgrad(const DeviceData<uint64_t> *A, const DeviceData<uint64_t> *B, DeviceData<uint64_t> *C, int b,
                       int deltaHeight, int deltaWidth, int Dout, int filterHeight, int filterWidth, int Din,
                       int paddingHeight, int paddingWidth, int stride, int dilation, int imageHeight, int imageWidth) {
    (void)deltaHeight;
    (void)deltaWidth;
    if (filterHeight != filterWidth || paddingHeight != paddingWidth || dilation != 1)
        throw piranha_gb300::Error(PG_ERR_UNSUPPORTED, "conv_dgrad: square filters, equal paddings, dilation 1");
    piranha_gb300::check(pg_conv_u64(piranha_gb300::context(), PG_CONV_DGRAD, b, imageHeight, imageWidth, Din, Dout,
                                      filterHeight, filterWidth, paddingHeight, stride, A->data(), B->data(),
                                      C->data()));
}
/* conv_wgrad (conv.cuh:470-490): A = dY, B = X (b, H, W, Din), C = dF (Dout, fh, fw, Din) */
inline void conv_wgrad(const DeviceData<uint64_t> *A, const DeviceData<uint64_t> *B, DeviceData<uint64_t> *C, int b,
                       int deltaHeight, int deltaWidth, int Dout, int imageHeight, int imageWidth, int Din,
                       int filterHeight, int filterWidth, int paddingHeight, int paddingWidth, int stride,
                       int dilation) {
    (void)deltaHeight;
    (void)deltaWidth;
    if (filterHeight != filterWidth || paddingHeight != paddingWidth || dilation != 1)
        throw piranha_gb300::Error(PG_ERR_UNSUPPORTED, "conv_wgrad: square filters, equal paddings, dilation 1");
    piranha_gb300::check(pg_conv_u64(piranha_gb300::context(), PG_CONV_WGRAD, b, imageHeight, imageWidth, Din, Dout,
                                      filterHeight, filterWidth, paddingHeight, stride, A->data(), B->data(),
                                      C->data()));
}

/* maxpool_im2row (convolution.cuh:252-304): the pools of every window,
 * padded with pad_val to the reference's padded pool size
 * pow(ceil(log2(f * f)), 2); output is resized to hold them */
template <typename U>
inline void maxpool_im2row(const DeviceData<uint64_t> *im, DeviceData<uint64_t> *output, int imageHeight,
                           int imageWidth, int filterSize, int Din, int batchSize, int stride, int padding,
                           U pad_val) {
    const int wk = (imageWidth - filterSize + 2 * padding) / stride + 1;
    const int hk = (imageHeight - filterSize + 2 * padding) / stride + 1;
    const int padded = (int)std::pow(std::ceil(std::log2((double)(filterSize * filterSize))), 2);
    output->resize((size_t)padded * wk * hk * batchSize * Din);
    piranha_gb300::check(pg_maxpool_im2row_u64(piranha_gb300::context(), im->data(), output->data(), imageHeight,
                                                imageWidth, filterSize, Din, batchSize, stride, padding,
                                                (uint64_t)(int64_t)pad_val));
}
/* the same on share i of every party (the reference's loop over getShare(i)) */
template <typename U>
inline void maxpool_im2row(SharePart<uint64_t> im, SharePart<uint64_t> output, int imageHeight, int imageWidth,
                           int filterSize, int Din, int batchSize, int stride, int padding, U pad_val) {
    const int wk = (imageWidth - filterSize + 2 * padding) / stride + 1;
    const int hk = (imageHeight - filterSize + 2 * padding) / stride + 1;
    const int padded = (int)std::pow(std::ceil(std::log2((double)(filterSize * filterSize))), 2);
    output.owner().resize((size_t)padded * wk * hk * batchSize * Din);
    for (int p = 0; p < 3; p++)
        piranha_gb300::check(pg_maxpool_im2row_u64(piranha_gb300::context(), im.party(p), output.party(p), imageHeight,
                                                    imageWidth, filterSize, Din, batchSize, stride, padding,
                                                    (uint64_t)(int64_t)pad_val));
}

/* truncate_cols (matrix.cuh:383-396): a holds rows of start_cols columns;
 * the first end_cols columns of each row go to b */
inline void truncate_cols(const DeviceData<uint8_t> *a, DeviceData<uint8_t> *b, size_t rows, size_t start_cols,
                          size_t end_cols) {
    piranha_gb300::check(pg_truncate_cols_u8(piranha_gb300::context(), a->data(), b->data(), rows, (int)start_cols,
                                             (int)end_cols));
}
inline void truncate_cols(SharePart<uint8_t> a, SharePart<uint8_t> b, size_t rows, size_t start_cols,
                          size_t end_cols) {
    for (int p = 0; p < 3; p++)
        piranha_gb300::check(pg_truncate_cols_u8(piranha_gb300::context(), a.party(p), b.party(p), rows,
                                                 (int)start_cols, (int)end_cols));
}

/* elementVectorAdd (matrix.cuh:75-84) and reduceSum (:109-126) */
inline void elementVectorAdd(DeviceData<uint64_t> *a, const DeviceData<uint64_t> *b, bool rowwise, int rows,
                             int cols) {
    piranha_gb300::check(pg_element_vector_add_u64(piranha_gb300::context(), a->data(), b->data(), rowwise, rows, cols));
}
inline void reduceSum(const DeviceData<uint64_t> *a, DeviceData<uint64_t> *b, bool reduceRows, int rows, int cols) {
    piranha_gb300::check(pg_reduce_sum_u64(piranha_gb300::context(), a->data(), b->data(), reduceRows, rows, cols));
}

}  // namespace gpu

#endif /* PIRANHA_GB300_HPP */
