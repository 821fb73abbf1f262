// func_kat.cpp — the reference's protocol known-answer tests (src/test/Func.cu,
// src/test/GPU.cu) written against the C++ share-class layer
// (include/piranha_gb300.hpp), the way the reference's own tests call RSS<T>,
// DeviceData<T>, matmul, dReLU, ReLU, maxpool, gpu::gemm and gpu::conv_fprop.
//
// Input (stdin), one case at a time:
//   case <Name>
//   arr <key> <n> <n doubles>      (zero or more)
//   param <key> <integer>          (zero or more)
//   run
// Output per case: the revealed results as doubles (party A's reconstruct,
// decoded from fixed point where the reference's test decodes them) and the
// six share buffers of each result tensor, for tests/test_gpu_cpp_layer.py to
// compare with the expected values and with the oracle.
#include <cstdio>
#include <iomanip>
#include <iostream>
#include <map>
#include <sstream>
#include <string>
#include <vector>

#include "piranha_gb300.hpp"

typedef uint64_t T;
typedef RSS<T> Share;

struct Case {
    std::string name;
    std::map<std::string, std::vector<double>> arr;
    std::map<std::string, long long> param;
};

static RSS<T> share_of(const std::vector<double> &v, bool fixed = true) {
    // the initializer-list constructor's semantics for a runtime list
    RSS<T> s(v.size());
    std::vector<T> x;
    for (double f : v) x.push_back(piranha_gb300::encode<T>(f, fixed));
    s.upload(0, 0, x);
    s.upload(2, 1, x);
    return s;
}

template <typename U> static void print_revealed(const std::string &c, const std::string &key, const RSS<U> &s,
                                                 bool fixed) {
    DeviceData<U> result(s.size());
    reconstruct(s, result);
    std::vector<U> h = result.download();
    std::cout << "out " << c << " " << key << " " << h.size();
    for (U v : h) {
        const double d = (double)(int64_t)(uint64_t)v;
        std::cout << " " << (fixed ? (double)(int64_t)v / (double)(1ull << FLOAT_PRECISION) : d);
    }
    std::cout << "\n";
}

template <typename U> static void print_shares(const std::string &c, const std::string &key, const RSS<U> &s) {
    std::cout << "shares " << c << " " << key << " " << s.size();
    for (int p = 0; p < 3; p++)
        for (int i = 0; i < 2; i++)
            for (U v : s.download(p, i)) std::cout << " " << (uint64_t)v;
    std::cout << "\n";
}

static void print_plain(const std::string &c, const std::string &key, const DeviceData<T> &d) {
    std::vector<T> h = d.download();
    std::cout << "plain " << c << " " << key << " " << h.size();
    for (T v : h) std::cout << " " << v;
    std::cout << "\n";
}

static void run(const Case &k) {
    const std::string &n = k.name;
    auto A = [&](const char *key) { return k.arr.at(key); };
    auto P = [&](const char *key) { return (int)k.param.at(key); };
    if (n == "Reconstruct") {
        Share a = share_of(A("a"));
        print_revealed(n, "result", a, true);
    } else if (n == "MatMul" || n == "MatMul2") {
        Share a = share_of(A("a")), b = share_of(A("b"));
        Share c((size_t)P("M") * P("N"));
        matmul(a, b, c, P("M"), P("N"), P("K"), P("tA"), P("tB"), P("tC"), (T)FLOAT_PRECISION);
        print_revealed(n, "result", c, true);
        print_shares(n, "c", c);
    } else if (n == "Mult") {
        Share a = share_of(A("a"), false), b = share_of(A("b"), false);
        b *= a;
        print_revealed(n, "result", b, false);
        print_shares(n, "b", b);
    } else if (n == "Truncate" || n == "Truncate2") {
        Share a = share_of(A("a"));
        dividePublic(a, (T)P("d"));
        print_revealed(n, "result", a, true);
        print_shares(n, "a", a);
    } else if (n == "TruncateVec") {
        Share a = share_of(A("a"));
        DeviceData<T> denominators(a.size());
        denominators.fill(1);
        std::vector<T> pw;
        for (double v : A("pows")) pw.push_back((T)v);
        DeviceData<T> pows(pw.size());
        pows.upload(pw);
        denominators <<= pows;
        dividePublic(a, denominators);
        print_revealed(n, "result", a, true);
        print_shares(n, "a", a);
    } else if (n == "SelectShare") {
        Share x = share_of(A("x")), y = share_of(A("y"));
        Share b = share_of(A("b"), false);
        Share z(x.size());
        selectShare(x, y, b, z);
        print_revealed(n, "result", z, true);
        print_shares(n, "z", z);
    } else if (n == "Convolution") {
        Share im = share_of(A("im")), filters = share_of(A("filters"));
        const int H = P("H"), W = P("W"), f = P("f"), pad = P("pad"), stride = P("stride");
        const int wk = (W - f + 2 * pad) / stride + 1, hk = (H - f + 2 * pad) / stride + 1;
        Share out((size_t)P("batch") * wk * hk * P("Dout"));
        convolution(im, filters, out, cutlass::conv::Operator::kFprop, P("batch"), H, W, f, P("Din"), P("Dout"),
                    stride, pad, FLOAT_PRECISION);
        print_revealed(n, "result", out, true);
        print_shares(n, "out", out);
    } else if (n == "DRELU" || n == "DRELU2" || n == "DRELU3") {
        Share input = share_of(A("input"));
        if (n == "DRELU3") {
            // -10 added to the last three values at every share of every party
            const T negative = (T)(-10 * (1 << FLOAT_PRECISION));
            DeviceData<T> add = {0, 0, 0, 0, 0, negative, negative, negative};
            for (int share = 0; share < Share::numShares(); share++) *input.getShare(share) += add;
        }
        Share result(input.size());
        dReLU(input, result);
        print_revealed(n, "result", result, false);
        print_shares(n, "result", result);
    } else if (n == "RELU") {
        Share input = share_of(A("input"));
        Share result(input.size()), dresult(input.size());
        ReLU(input, result, dresult);
        print_revealed(n, "result", result, true);
        print_revealed(n, "dresult", dresult, false);
        print_shares(n, "result", result);
    } else if (n == "Maxpool") {
        Share input = share_of(A("input"));
        const int kk = P("k");
        Share result(input.size() / kk), dresult(input.size());
        maxpool(input, result, dresult, kk);
        print_revealed(n, "result", result, true);
        print_revealed(n, "dresult", dresult, false);
        print_shares(n, "result", result);
    } else if (n == "Maxpool2") {
        // gpu::maxpool_im2row over a 3x3 pool padded to 16, maxpool, then
        // gpu::truncate_cols of the derivative back to the 9 pool columns
        Share input = share_of(A("input"));
        Share result(1);
        RSS<uint8_t> dresult(input.size());
        const int expandedPoolSize = 16;
        Share pools((size_t)0);
        for (int share = 0; share < Share::numShares(); share++)
            gpu::maxpool_im2row(input.getShare(share), pools.getShare(share), 3, 3, 3, 1, 1, 1, 0, -10);
        RSS<uint8_t> expandedMaxPrime(pools.size());
        maxpool(pools, result, expandedMaxPrime, expandedPoolSize);
        for (int share = 0; share < Share::numShares(); share++)
            gpu::truncate_cols(expandedMaxPrime.getShare(share), dresult.getShare(share),
                               pools.size() / expandedPoolSize, expandedPoolSize, 9);
        print_revealed(n, "result", result, true);
        print_revealed(n, "dresult", dresult, false);
        print_shares(n, "result", result);
    } else if (n == "CutlassGemm") {
        std::vector<T> ha, hb;
        for (double v : A("a")) ha.push_back((T)(int64_t)v);
        for (double v : A("b")) hb.push_back((T)(int64_t)v);
        DeviceData<T> a(ha.size()), b(hb.size()), c((size_t)P("M") * P("N"));
        a.upload(ha);
        b.upload(hb);
        gpu::gemm(P("M"), P("N"), P("K"), &a, P("tA"), &b, P("tB"), &c, P("tC"));
        print_plain(n, "c", c);
    } else if (n == "CutlassConvFprop") {
        std::vector<T> hi, hf;
        for (double v : A("im")) hi.push_back((T)(int64_t)v);
        for (double v : A("f")) hf.push_back((T)(int64_t)v);
        const int N = P("N"), H = P("H"), W = P("W"), C = P("C"), K = P("K"), R = P("R"), pad = P("pad"),
                  st = P("stride");
        const int Pp = (H + 2 * pad - R) / st + 1, Q = (W + 2 * pad - R) / st + 1;
        DeviceData<T> im(hi.size()), fl(hf.size()), out((size_t)N * Pp * Q * K);
        im.upload(hi);
        fl.upload(hf);
        gpu::conv_fprop(&im, &fl, &out, N, H, W, C, K, R, R, pad, pad, st, 1);
        print_plain(n, "out", out);
    } else {
        throw piranha_gb300::Error(PG_ERR_INVALID_ARG, "unknown case " + n);
    }
}

int main() {
    std::cout << std::setprecision(17);
    std::string line;
    Case k;
    int status = 0;
    while (std::getline(std::cin, line)) {
        std::istringstream in(line);
        std::string tag;
        in >> tag;
        if (tag == "case") {
            k = Case();
            in >> k.name;
        } else if (tag == "arr") {
            std::string key;
            size_t cnt;
            in >> key >> cnt;
            std::vector<double> v(cnt);
            for (size_t i = 0; i < cnt; i++) in >> v[i];
            k.arr[key] = v;
        } else if (tag == "param") {
            std::string key;
            long long v;
            in >> key >> v;
            k.param[key] = v;
        } else if (tag == "run") {
            try {
                run(k);
            } catch (const std::exception &e) {
                std::cout << "error " << k.name << " " << e.what() << "\n";
                status = 1;
            }
        }
    }
    int code = 0;
    pg_device_errors(piranha_gb300::context(), &code);
    if (code) {
        std::cout << "error device " << code << "\n";
        status = 1;
    }
    pg_ctx_destroy(piranha_gb300::context());
    return status;
}
