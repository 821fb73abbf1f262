// pg_limb_tma.cuh — host-side plan of the TMA-fed limb tensor-core share-GEMM
// (pg_limb_tma.cu): problem geometry, the digit-plane image of A, the packed
// weights, the tile rectangle, and the three launches (image, pack, GEMM).
#pragma once

#include <stddef.h>
#include <stdint.h>

#include <string>

namespace pg {
struct Ctx;
namespace lt {

struct Plan {
    int implicit;       // 1: image = activation tensor (taps are box shifts); 0: one image row per output row
    int src_mode;       // how the image kernel reads A (rows, columns, im2col gather)
    long long ld;       // row / column stride of A for rows / columns
    long long pixels;   // image rows that come from A
    long long pixels_alloc;  // image rows stored (a whole number of 32-row lines for the GEMM form)
    int C;              // image channels (multiple of 16)
    int Kreal;          // real channels of A per image row (image channels >= Kreal are 0)
    int Wimg, Himg, Nimg;  // image tensor extents (W, H, images) seen by the tensor map
    int H, W, Din, stride; // input geometry of a convolution
    int cf, cpad, cP, cQ;  // convolution taps, padding and output extents for the im2col gather
    int f, pad, P, Q;      // taps and output extents the GEMM kernel iterates (1, 0, 1, 1 unless implicit)
    int M, N, kblocks, cblocks, ntiles_n;
    int Wt, Ht, Nt, R, tiles_w, tiles_h, tiles_m;  // output-pixel rectangle of a tile, rows used
    int tB_kn;          // weights as b[k * N + n] (1) or b[n * Kb + k] (0)
    int colmajor;       // output column-major (GEMM with tC = 0)
    int posmajor;       // implicit convolution tiled by output position: a tile is one output pixel (p, q) of
                        // 128 images, the image is stored batch-innermost (pixel (h * W + w) * Nimg + n), and
                        // the tile runs only the taps that fall inside the input (no zero-padding taps)
    int C8;             // wgt: image channels (Din, or Din rounded up to 8 when below 128)
    int flip_f;         // > 0: the input gradient as a convolution of dY with the flipped filter (f x f, B = W[Dout]
                        // [f][f][Din] read at tap (f-1-r, f-1-s) and transposed); 0: the weights as given
    int wgt;            // implicit weight gradient: rows (tap, c), K = output pixels x images (16 per stage);
                        // the image is the forward input as [seg][plane][h * W + w][n / 8][c][n % 8], a tile
                        // is 128 channels of one tap and runs only the output pixels whose tap lands inside
    size_t image_bytes, packB_bytes;
};

int prepare_device(Ctx *c, bool again = false);  // once per device (again: repeat it), with it current (no allocation)
int plan_gemm(Ctx *c, Plan &p, int M, int N, int K, int tA, int tB, int tC);
// posmajor_ok = false: rectangle tiles even where position-major ones apply
int plan_conv(Ctx *c, Plan &p, int batch, int H, int W, int f, int Din, int Dout, int stride, int pad,
              bool posmajor_ok = true);
// the weight gradient of that convolution as a GEMM over the output pixels
// implicit_ok = false: the explicit transposed-im2col image even where the implicit form applies
int plan_wgrad(Ctx *c, Plan &p, int batch, int H, int W, int f, int Din, int Dout, int stride, int pad,
               bool implicit_ok = true);
// whether the implicit weight gradient applies (stride 1, a multiple of 16 images)
bool wgrad_implicit_applies(int batch, int stride);
// the input gradient of a stride-1 convolution as an implicit convolution of dY (P x Q x Dout, padded by
// f - 1 - pad) with the flipped, transposed filter; PG_ERR_UNSUPPORTED where that is not an implicit plan
int plan_dgrad_flip(Ctx *c, Plan &p, int batch, int H, int W, int f, int Din, int Dout, int stride, int pad);
void choose_split(const Plan &p, int sms, int &split, int &chunks_per_split);
size_t partial_bytes(const Plan &p, int split);
// the split-K autotuner: partial bytes that every candidate fits in, and the
// choice (cached per shape in the context; timed when the context allows)
size_t tune_partial_bytes(const Plan &p, int sms);
bool cached_split(Ctx *c, const Plan &p, int &split, int &chunks_per_split);
// the shape key of a plan in the context's tuning cache
std::string plan_key(const Plan &p);
int tune_split(Ctx *c, const Plan &p, const void *image, const void *packB, uint64_t *partial,
               uint64_t *const out[6], const uint64_t *const bias[6], int trunc, bool zeros_kept, uint64_t *raw,
               int &split, int &chunks_per_split, bool shared = false);
// A shares -> digit-plane image; weight shares -> packed stage images; then the GEMM (+ split-K reduction).
// shared (run_image, run_relu_image, run_gemm): the six share buffers hold a replicated sharing (party p's
// second share equals party p+1's first, bit for bit), so the image stores each of the three shares once
// (block b = party b's first share) and the GEMM reads segment s (party s/2's share s%2) from block
// ((s + 1) / 2) % 3; the image producer and the GEMM must agree on it.
// rep_flag (run_image, run_gemm): a device word, set where a[]'s buffers hold a replicated sharing (checked on
// the device by the caller); the image kernel and the GEMM then use the three-block layout
int run_image(Ctx *c, const Plan &p, const uint64_t *const a[6], void *image, bool shared = false,
              const int *rep_flag = nullptr);
int run_pack(Ctx *c, const Plan &p, const uint64_t *const b[6], void *packB);
// ReLU of n values fused with the digit image of the implicit convolution
// (plan p) that takes them as input; relu_image_fits says whether it applies.
// out == nullptr: the ReLU output is kept in the image alone; dout == nullptr:
// no bit shares (an inference forward needs neither)
bool relu_image_fits(const Plan &p, size_t n);
int run_relu_image(Ctx *c, const Plan &p, const uint64_t *const in[6], size_t n, uint64_t *const out[6],
                   uint8_t *const dout[6], void *image, bool shared = false);
// the six u64 shares of the n values that run_relu_image left in image (plan p, the same shared)
int run_image_decode(Ctx *c, const Plan &p, const void *image, size_t n, uint64_t *const out[6], bool shared);
// zeros_kept: the four output shares that dividePublic3out3 leaves at 0 (all
// but party A's shareA and party C's shareB) already hold 0 and are only
// written where a bias share is added (the network's zeroed arena).
// raw: write the untruncated Z (M x N, row-major) there instead of shares.
int run_gemm(Ctx *c, const Plan &p, const void *image, const void *packB, uint64_t *partial, int split,
             int chunks_per_split, uint64_t *const out[6], const uint64_t *const bias[6], int trunc,
             bool zeros_kept = false, uint64_t *raw = nullptr, bool shared = false, const int *rep_flag = nullptr);

}  // namespace lt
}  // namespace pg
