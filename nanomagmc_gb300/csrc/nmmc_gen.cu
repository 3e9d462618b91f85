// Learned warm start: a conditional convolutional generator for 2-D Heisenberg lattices.
//
// No reference counterpart. The plain sampler produces equilibrium snapshots x at points
// c = (T, B, D); the network learns to denoise y = normalise(sqrt(1-s^2) x + s g) (g standard
// normal per site and component, s the noise level; at s = 1, y is a uniform random start)
// back to x. A warm start runs a few denoising steps from a random start and hands the
// result to the Metropolis chain, which does all sampling.
//
// Network: 8 periodic 3x3 convolutions, 48 channels, ReLU between layers. Input channels:
// y (3), T/1.5, B, D/0.8, s, 0. Output: 3 channels v, spin = v/|v|. Loss: mean over sites of
// |v/|v| - x|^2. Weights and activations are stored in BF16, every product is accumulated in
// FP32; gradients, biases, master weights and the Adam moments are FP32.
//
// Layouts: activations NHWC [image][y][x][channel]; weights [tap = 3*(dy+1)+(dx+1)][cin][cout].
#include <cuda.h>
#include <cuda_bf16.h>
#include <math.h>
#include <stdio.h>
#include <string.h>

#include <algorithm>
#include <map>
#include <vector>

#include "nmmc_internal.h"

namespace nmmc {

constexpr int kGenC = 48;        // hidden channels
constexpr int kGenLayers = 8;
constexpr int kGenCin0 = 8;      // 3 spin + 4 condition + 1 zero
constexpr int kGenCout = 4;      // 3 spin components + 1 zero (vector loads)
constexpr int kWimgBytes = 9 * (kGenC / 8) * (kGenC / 8) * 128;   // largest layer weight image (48 -> 48)
constexpr int kTile = 16;        // pixel tile edge of the convolution kernels

// Activations and gradients are stored chunk-planar: C channels of element type T as
// [image][C / epc][L*L pixels][epc], epc = 16 / sizeof(T) (8 BF16 or 4 FP32 channels per
// 16-byte chunk), so that a chunk of consecutive pixels of a row is contiguous: one TMA box
// per (row, chunk) of a convolution window and coalesced stores. A tensor of a single chunk
// (the 8-channel input, the 4-channel output and its gradient) is plain [pixel][C].
template <typename T>
__host__ __device__ constexpr int epc() { return 16 / (int)sizeof(T); }
// element offset of channel c of pixel pp (y*L + x) of image img
template <typename T>
__host__ __device__ __forceinline__ size_t pl_off(int C, size_t LL, size_t img, size_t pp, int c) {
    return ((img * (size_t)(C / epc<T>()) + (size_t)(c / epc<T>())) * LL + pp) * (size_t)epc<T>() + (size_t)(c % epc<T>());
}

struct GenLayer {
    int cin = 0, cout = 0;           // cout padded to kGenCout for the last layer
    float* w = nullptr;              // FP32 master [9][cin][cout]
    float* b = nullptr;              // [cout]
    __nv_bfloat16* wb = nullptr;     // BF16 compute copy [9][cin][cout]
    __nv_bfloat16* wt = nullptr;     // BF16 flipped transpose [9][cout][cin] (data gradient)
    uint8_t* wimg = nullptr;         // BF16 weights in the tensor-core B layout of k_gen_conv_tma
                                     // (kWimgBytes), staged by one bulk copy per CTA
    float* gw = nullptr;
    float* gb = nullptr;
    float* mw = nullptr;
    float* vw = nullptr;
    float* mb = nullptr;
    float* vb = nullptr;
    size_t nw() const { return (size_t)9 * cin * cout; }
};

}  // namespace nmmc

struct nmmc_gen {
    int L = 0;
    uint64_t seed = 0;
    cudaStream_t stream = nullptr;
    nmmc::GenLayer layer[nmmc::kGenLayers];
    // dataset
    int cap = 0, count = 0;
    __nv_bfloat16* snaps = nullptr;  // [cap][L][L][3]
    float* cond = nullptr;           // [cap][3]
    // batch workspace
    int bcap = 0;
    __nv_bfloat16* act[nmmc::kGenLayers] = {};   // act[0] input (8 ch); act[l] output of layer l-1,
                                                 // [b][6][L][L][8] (chunk-planar)
    float* vout = nullptr;           // [b][L][L][4] linear output of the last layer
    float* target = nullptr;         // [b][L][L][4]
    float* g0 = nullptr;             // gradient ping-pong [b][12][L][L][4] (chunk-planar)
    float* g1 = nullptr;
    float* gv = nullptr;             // [b][L][L][4]
    float* wpart = nullptr;          // weight-gradient partials
    size_t wpart_cap = 0;
    int* d_idx = nullptr;            // snapshot index per batch item
    float* d_sig = nullptr;          // noise level per batch item
    float* d_cnd = nullptr;          // condition per batch item (3)
    double* d_loss = nullptr;
    int* d_flag = nullptr;           // device error word (4: a tensor-core wait gave up)
    int use_tc = 1;                  // hidden layers on tcgen05 (NMMC_GEN_OPT_TENSOR_CORES)
    int use_ws = 0;                  // warp-specialised tcgen05 kernel for the BF16 modes (opt-in)
    int use_tma = 1;                 // L = 128: 1 TMA-staged single-role kernels, 2 TMA-staged
                                     // warp-specialised forward, 0 cp.async staging
    int tile_rows = 2;               // output rows per tile of the TMA forward kernels (1 or 2)
    int schedule = 0;                // warm-start noise levels: 0 linear, 1 quadratic, 2 cosine
    int use_wimg = 1;                // TMA forward kernels stage the weights by one bulk copy of
                                     // their image (0: the threads rearrange the BF16 weights)
    int sm_count = 0;
    int smem_per_sm = 0;             // shared memory per SM of the generator's device
    std::map<const void*, int> attr_smem;   // dynamic shared memory set per kernel on that device
    long long adam_t = 0;
    unsigned long long draws = 0;    // Philox counter for noise
};

namespace nmmc {

// ------------------------------------------------------------------------------------------
// Convolution (forward and data gradient share it): out[p, co] = sum_{tap, ci} in[p + tap, ci] *
// W[tap][ci][co] (+ bias), periodic in x and y. One CTA = one 16x16 pixel tile of one image;
// 256 threads = 128 pixel pairs (rows y and y+8) x 2 halves of the output channels.
// EPI 0: ReLU, BF16 out.  EPI 1: linear, FP32 out.  EPI 2: times (mask > 0), FP32 out.
// ------------------------------------------------------------------------------------------
template <int CIN, int COUT, typename TIN, int EPI>
__global__ void __launch_bounds__(256)
k_gen_conv(const TIN* __restrict__ in, const __nv_bfloat16* __restrict__ w, const float* __restrict__ bias,
           const __nv_bfloat16* __restrict__ mask, int mask_c, void* __restrict__ out, int L) {
    extern __shared__ float gsm[];
    constexpr int HALF = (COUT + 1) / 2;          // output channels per thread
    constexpr int T2 = kTile + 2;
    float* wsm = gsm;                              // [9][CIN][COUT]
    float* tsm = gsm + 9 * CIN * COUT;             // [CIN][T2][T2]
    const int img = blockIdx.z;
    const int ty0 = blockIdx.y * kTile, tx0 = blockIdx.x * kTile;
    // weights and the wrapped input tile through 16-byte loads, several in flight per thread
    // (weight arrays and pixel rows are 16-byte multiples and the buffers 16-byte aligned)
    static_assert((9 * CIN * COUT) % 8 == 0 && (CIN * sizeof(TIN)) % 16 == 0, "16-byte staging");
#pragma unroll 4
    for (int i = threadIdx.x; i < 9 * CIN * COUT / 8; i += blockDim.x) {
        const uint4 q = __ldg(reinterpret_cast<const uint4*>(w) + i);
        const __nv_bfloat16* e = reinterpret_cast<const __nv_bfloat16*>(&q);
#pragma unroll
        for (int k = 0; k < 8; ++k) wsm[8 * i + k] = __bfloat162float(e[k]);
    }
    const size_t LL = (size_t)L * L, ibase = (size_t)img * LL;
    constexpr int EPV = epc<TIN>(), V = CIN / EPV;   // elements per load, chunks per pixel
    const uint4* src = reinterpret_cast<const uint4*>(in + ibase * CIN);   // this image's chunk planes
#pragma unroll 4
    for (int i = threadIdx.x; i < T2 * T2 * V; i += blockDim.x) {   // x fastest: coalesced rows
        const int v = i / (T2 * T2), r = i - v * T2 * T2, yy = r / T2, xx = r - yy * T2;
        int gy = ty0 + yy - 1, gx = tx0 + xx - 1;   // in [-1, L]: one wrap
        gy += (gy < 0) ? L : ((gy >= L) ? -L : 0);
        gx += (gx < 0) ? L : ((gx >= L) ? -L : 0);
        const uint4 q = __ldg(src + (size_t)v * LL + (size_t)gy * L + gx);
        const TIN* e = reinterpret_cast<const TIN*>(&q);
#pragma unroll
        for (int k = 0; k < EPV; ++k) tsm[((v * EPV + k) * T2 + yy) * T2 + xx] = (float)e[k];
    }
    __syncthreads();
    const int pair = threadIdx.x & 127, half = threadIdx.x >> 7;
    const int px = pair & 15, py = pair >> 4;      // rows py and py + 8
    const int co0 = half * HALF;
    float a0[HALF], a1[HALF];
#pragma unroll
    for (int k = 0; k < HALF; ++k) {
        const int co = co0 + k;
        const float bv = (bias && co < COUT) ? bias[co] : 0.0f;
        a0[k] = bv;
        a1[k] = bv;
    }
#pragma unroll 1
    for (int tap = 0; tap < 9; ++tap) {
        const int dy = tap / 3, dx = tap - 3 * (tap / 3);
#pragma unroll 4
        for (int ci = 0; ci < CIN; ++ci) {
            const float x0 = tsm[(ci * T2 + py + dy) * T2 + px + dx];
            const float x1 = tsm[(ci * T2 + py + 8 + dy) * T2 + px + dx];
            const float* wr = wsm + (tap * CIN + ci) * COUT + co0;
#pragma unroll
            for (int k = 0; k < HALF; ++k) {
                if (co0 + k < COUT) {
                    a0[k] = fmaf(x0, wr[k], a0[k]);
                    a1[k] = fmaf(x1, wr[k], a1[k]);
                }
            }
        }
    }
#pragma unroll
    for (int r = 0; r < 2; ++r) {
        const int y = ty0 + py + 8 * r, x = tx0 + px;
        const size_t pp = (size_t)y * L + x;
        const float* a = r ? a1 : a0;
#pragma unroll
        for (int k = 0; k < HALF; ++k) {
            const int co = co0 + k;
            if (co >= COUT) continue;
            float v = a[k];
            if (EPI == 0) {
                ((__nv_bfloat16*)out)[pl_off<__nv_bfloat16>(COUT, LL, img, pp, co)] = __float2bfloat16(fmaxf(v, 0.0f));
            } else if (EPI == 1) {
                ((float*)out)[pl_off<float>(COUT, LL, img, pp, co)] = v;
            } else {
                const float mk = __bfloat162float(mask[pl_off<__nv_bfloat16>(mask_c, LL, img, pp, co)]);
                ((float*)out)[pl_off<float>(COUT, LL, img, pp, co)] = mk > 0.0f ? v : 0.0f;
            }
        }
    }
}

// ------------------------------------------------------------------------------------------
// Hidden-layer convolutions (48 -> 48 channels) on the 5th-generation tensor cores, as an
// implicit GEMM over the periodically padded image: with rows of pitch L+2 (one wrapped
// column each side), output position P of the padded grid is sum_tap in[P + off_tap] W_tap,
// off_tap = (dy-1)(L+2) + (dx-1), so every tap is one shifted window of the same staged
// data. A tile is 128 consecutive padded positions of rows 1..L (one TMEM lane each; halo
// positions are computed and dropped), N = 48 output channels (FP32 TMEM columns), K = 9 taps
// x 48 input channels, 32 bytes of K per MMA.
//
//   MODE 0 (forward):  BF16 activations, tcgen05.mma kind::f16; bias + ReLU, BF16 out.
//   MODE 1 (probe):    as 0 with bias only and FP32 out.
//   MODE 2 (data gradient): FP32 gradients as TF32 operands (kind::tf32) with the flipped,
//                      transposed weights; out = result x (activation > 0), FP32.
//
// Shared-memory operands use the K-major layout without swizzling, 8-row x 16-byte core
// matrices. The staged input window (W = 128 + 2(L+3) padded positions, wrapped while
// loading) is stored chunk-major: the 16-byte atom of chunk c (8 BF16 or 4 FP32 channels) of
// window position w at (c*W + w)*16, so a core matrix is 8 consecutive positions (stride byte
// offset 128 B), the next chunk is W*16 B further (leading byte offset), and a tap's window
// starts 16 B per position of its offset later. The layer's weights are staged once per CTA
// (persistent CTAs). One thread issues the MMAs of a tile and commits them to an mbarrier;
// after a bounded wait, each warp reads its 32 TMEM lanes (tcgen05.ld) for the epilogue.
// ------------------------------------------------------------------------------------------
namespace tc {
constexpr int kM = 128;                         // padded positions per tile = TMEM lanes
constexpr int kC = 48;                          // channels in and out
constexpr int kCore = 128;                      // bytes per core matrix
constexpr int kTmemCols = 64;                   // power of two >= 48
constexpr unsigned kWaitLimit = 1u << 26;

template <int MODE>
struct Traits {
    using TA = __nv_bfloat16;                   // operand element type
    static constexpr int kEpc = 8;              // elements per 16-byte chunk
    static constexpr uint32_t kFmt = 1;         // BF16
};
template <>
struct Traits<2> {
    using TA = float;
    static constexpr int kEpc = 4;
    static constexpr uint32_t kFmt = 2;         // TF32
};
template <int MODE>
__host__ __device__ constexpr int chunks() { return kC / Traits<MODE>::kEpc; }        // 6 (BF16) or 12 (TF32)
template <int MODE>
__host__ __device__ constexpr int btap() { return (kC / 8) * chunks<MODE>() * kCore; } // weight bytes per tap
// instruction descriptor: D F32 (bits 4-5 = 1), A and B format (bits 7-9, 10-12), both
// K-major (bits 15, 16 = 0), N >> 3 at bits 17-22, M >> 4 at bits 24-28
template <int MODE, int N = kC>
__host__ __device__ constexpr uint32_t idesc() {
    return (1u << 4) | (Traits<MODE>::kFmt << 7) | (Traits<MODE>::kFmt << 10) | ((uint32_t)(N >> 3) << 17) |
           ((uint32_t)(kM >> 4) << 24);
}
__host__ __device__ constexpr int window(int L) { return kM + 2 * (L + 3); }
template <int MODE>
__host__ __device__ constexpr int smem_bytes(int L) { return 9 * btap<MODE>() + chunks<MODE>() * window(L) * 16 + 1024; }
constexpr int kSmemMax = 232448;                // dynamic shared memory per block (227 KB)
}  // namespace tc

__device__ __forceinline__ uint32_t gen_smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

// Shared-memory matrix descriptor: start address, leading and stride byte offsets (all >> 4),
// descriptor version 1 (bit 46), no swizzle (bits 61-63 = 0).
__device__ __forceinline__ uint64_t umma_desc(uint32_t addr, uint32_t lbo, uint32_t sbo) {
    return (uint64_t)((addr >> 4) & 0x3FFFu) | ((uint64_t)((lbo >> 4) & 0x3FFFu) << 16) |
           ((uint64_t)((sbo >> 4) & 0x3FFFu) << 32) | (1ull << 46);
}

__device__ __forceinline__ bool gen_mbar_try_wait(uint32_t bar, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(bar), "r"(parity)
        : "memory");
    return ok != 0;
}

// 16 consecutive FP32 columns of this thread's TMEM lane.
__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float* v) {
    uint32_t r[16];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, "
        "%14, %15}, [%16];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
          "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
        : "r"(taddr));
#pragma unroll
    for (int i = 0; i < 16; ++i) v[i] = __uint_as_float(r[i]);
}

// Weights w[tap][k][n] (BF16, 16-byte aligned) -> B_tap[n][k] as K-major core matrices in
// shared memory. One 16-byte load brings 8 consecutive n (48 is a multiple of 8) and the loop
// is unrolled so that several loads are in flight per thread; element by element, the loads
// would each wait for the previous store.
template <int MODE>
__device__ __forceinline__ void stage_weights(uint8_t* sB, const __nv_bfloat16* __restrict__ w, int tid, int nthr) {
    using TA = typename tc::Traits<MODE>::TA;
    constexpr int kEpc = tc::Traits<MODE>::kEpc, kCh = tc::chunks<MODE>(), kBT = tc::btap<MODE>();
    constexpr int kC = tc::kC, kG = 9 * kC * kC / 8;
#pragma unroll 7
    for (int g8 = tid; g8 < kG; g8 += nthr) {
        const uint4 v = __ldg(reinterpret_cast<const uint4*>(w) + g8);
        const int i = g8 * 8;
        const int tap = i / (kC * kC), r = i - tap * kC * kC, k = r / kC, n = r - k * kC;
        uint8_t* base = sB + tap * kBT + ((n >> 3) * kCh + k / kEpc) * tc::kCore + (k % kEpc) * (int)sizeof(TA);
        const __nv_bfloat16* e = reinterpret_cast<const __nv_bfloat16*>(&v);
#pragma unroll
        for (int q = 0; q < 8; ++q) *(TA*)(base + q * 16) = (TA)e[q];
    }
}

// Epilogue of one output position of a tensor-core convolution: v[48] FP32 accumulators of
// pixel pp (y*L + x) of image img, written chunk-planar (16 bytes per chunk, consecutive
// pixels of a warp contiguous). MODE 0: bias + ReLU, BF16. MODE 1: bias, FP32. MODE 2:
// times (mask > 0) with the mask the layer's BF16 activation, FP32.
template <int MODE>
__device__ __forceinline__ void conv_store(const float* v, const float* sbias, void* out_v,
                                           const __nv_bfloat16* __restrict__ mask, size_t img, size_t pp, size_t LL) {
    constexpr int kC = tc::kC;
    if (MODE == 0) {
        uint4* dst = reinterpret_cast<uint4*>((__nv_bfloat16*)out_v + img * LL * kC) + pp;
#pragma unroll
        for (int c = 0; c < kC / 8; ++c) {
            uint32_t h[4];
#pragma unroll
            for (int q = 0; q < 4; ++q) {
                const __nv_bfloat162 b2 = __floats2bfloat162_rn(fmaxf(v[8 * c + 2 * q] + sbias[8 * c + 2 * q], 0.0f),
                                                                fmaxf(v[8 * c + 2 * q + 1] + sbias[8 * c + 2 * q + 1], 0.0f));
                h[q] = *(const uint32_t*)&b2;
            }
            dst[(size_t)c * LL] = make_uint4(h[0], h[1], h[2], h[3]);
        }
    } else if (MODE == 1) {
        float4* dst = reinterpret_cast<float4*>((float*)out_v + img * LL * kC) + pp;
#pragma unroll
        for (int c = 0; c < kC / 4; ++c)
            dst[(size_t)c * LL] = make_float4(v[4 * c] + sbias[4 * c], v[4 * c + 1] + sbias[4 * c + 1],
                                              v[4 * c + 2] + sbias[4 * c + 2], v[4 * c + 3] + sbias[4 * c + 3]);
    } else {
        const uint4* mk = reinterpret_cast<const uint4*>(mask + img * LL * kC) + pp;
        float4* dst = reinterpret_cast<float4*>((float*)out_v + img * LL * kC) + pp;
#pragma unroll
        for (int c = 0; c < kC / 8; ++c) {
            const uint4 m4 = __ldg(mk + (size_t)c * LL);
            const __nv_bfloat16* mh = reinterpret_cast<const __nv_bfloat16*>(&m4);
            float o[8];
#pragma unroll
            for (int k = 0; k < 8; ++k) o[k] = (__bfloat162float(mh[k]) > 0.0f) ? v[8 * c + k] : 0.0f;
            dst[(size_t)(2 * c) * LL] = make_float4(o[0], o[1], o[2], o[3]);
            dst[(size_t)(2 * c + 1) * LL] = make_float4(o[4], o[5], o[6], o[7]);
        }
    }
}

template <int MODE, int N = tc::kC>
__device__ __forceinline__ void tc_mma(uint32_t tmem, uint64_t ad, uint64_t bd, uint32_t acc) {
    if (MODE == 2)
        asm volatile(
            "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
            "tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n\t}" ::"r"(tmem),
            "l"(ad), "l"(bd), "r"(tc::idesc<MODE, N>()), "r"(acc)
            : "memory");
    else
        asm volatile(
            "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
            "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(tmem),
            "l"(ad), "l"(bd), "r"(tc::idesc<MODE, N>()), "r"(acc)
            : "memory");
}

// Per tile: stage the window, issue the MMAs, wait for their commit, run the epilogue; two
// CTAs per SM overlap one another's phases. (Measured on GB300: a double-buffered variant with
// two accumulators, which fits one CTA per SM, and issuing the next tile's loads before the
// epilogue were both slower.)
template <int MODE>
__global__ void __launch_bounds__(128, 2)
k_gen_conv_tc(const typename tc::Traits<MODE>::TA* __restrict__ in, const __nv_bfloat16* __restrict__ w,
              const float* __restrict__ bias, const __nv_bfloat16* __restrict__ mask, void* __restrict__ out_v,
              int L, int tiles_per_img, int ntiles, int* __restrict__ flag) {
    using namespace tc;
    using TA = typename Traits<MODE>::TA;
    constexpr int kCh = chunks<MODE>();
    constexpr int kBT = btap<MODE>();
    constexpr int kRound = 96 / kCh;            // window positions per loader round (96 threads)
    extern __shared__ uint8_t tsm_raw[];
    __shared__ __align__(8) unsigned long long mbar;
    __shared__ uint32_t tmem_slot;
    __shared__ __align__(16) float sbias[kC];
    uint8_t* sB = (uint8_t*)(((uintptr_t)tsm_raw + 1023) & ~(uintptr_t)1023);
    uint8_t* sA = sB + 9 * kBT;
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int P = L + 2;                      // padded row pitch
    const int W = window(L);                  // staged window positions
    const int npad = P * P;

    // weights w[tap][k][n] (k: input channel of this convolution) -> B_tap[n][k], K-major
    stage_weights<MODE>(sB, w, tid, blockDim.x);
    if (tid < kC) sbias[tid] = (MODE == 2) ? 0.0f : bias[tid];
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(gen_smem_u32(&tmem_slot)),
                     "r"(kTmemCols)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    if (tid == 0) {
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(gen_smem_u32(&mbar)) : "memory");
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const uint32_t tmem = tmem_slot;
    const uint32_t aBase = gen_smem_u32(sA), bBase = gen_smem_u32(sB);

    // staged window of tile t into buffer buf: padded position w0 + j, wrapped onto the image;
    // outside the padded grid (only read by dropped halo outputs) zero. cp.async: every copy
    // of a thread is in flight at once. Threads 0..95 = kRound positions x kCh chunks per
    // round; a thread's padded row and column advance by kRound per round (P >= kRound).
    auto load_window = [&](int t) {
        const int img = t / tiles_per_img;
        const int w0 = (t - img * tiles_per_img) * kM - 1;        // q0 - (P + 1), q0 = P + tile*kM
        const TA* src_img = in + (size_t)img * L * L * kC;
        if (tid < kRound * kCh) {
            const int c = tid % kCh;
            int j = tid / kCh, pos = w0 + j;
            int py = (pos >= 0) ? pos / P : -1;
            int px = pos - py * P;
            const uint32_t dst0 = aBase + (uint32_t)(c * W * 16);
            for (; j < W; j += kRound, pos += kRound) {
                const bool inside = pos >= 0 && pos < npad;
                const uint4* src = (const uint4*)src_img;
                if (inside) {
                    int y = py - 1, x = px - 1;
                    y += (y < 0) ? L : ((y >= L) ? -L : 0);
                    x += (x < 0) ? L : ((x >= L) ? -L : 0);
                    src = (const uint4*)src_img + ((size_t)c * L * L + (size_t)y * L + x);   // chunk plane c
                }
                asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;" ::"r"(dst0 + (uint32_t)(j * 16)), "l"(src),
                             "r"(inside ? 16 : 0)
                             : "memory");
                px += kRound;
                if (px >= P) {
                    px -= P;
                    ++py;
                }
            }
        }
    };
    // the 9 x kCh/2 MMAs of a tile (thread 0), committed to the mbarrier
    auto issue_mmas = [&]() {
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        const uint32_t a0 = aBase, d = tmem;
#pragma unroll 1
        for (int tap = 0; tap < 9; ++tap) {
            const int shift = (P + 1) + (tap / 3 - 1) * P + (tap % 3 - 1);   // window slot of output 0
#pragma unroll
            for (int ks = 0; ks < kCh / 2; ++ks) {
                const uint64_t ad = umma_desc(a0 + (uint32_t)((2 * ks * W + shift) * 16), (uint32_t)(W * 16), 128);
                const uint64_t bd = umma_desc(bBase + tap * kBT + 2 * ks * kCore, kCore, kCh * kCore);
                tc_mma<MODE>(d, ad, bd, (tap | ks) ? 1u : 0u);
            }
        }
        asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                         gen_smem_u32(&mbar))
                     : "memory");
    };
    // epilogue of tile t: warp w holds positions q0 + 32w .. in TMEM lanes 32w ..
    auto epilogue = [&](int t) {
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        const int img = t / tiles_per_img;
        const int q0 = P + (t - img * tiles_per_img) * kM;
        float v[kC];
        const uint32_t taddr = tmem + ((uint32_t)(warp * 32) << 16);
        tmem_ld16(taddr + 0, v);
        tmem_ld16(taddr + 16, v + 16);
        tmem_ld16(taddr + 32, v + 32);
        asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
        const int pos = q0 + warp * 32 + lane, py = pos / P, px = pos - py * P;
        if (py >= 1 && py <= L && px >= 1 && px <= L) {
            conv_store<MODE>(v, sbias, out_v, mask, (size_t)img, (size_t)(py - 1) * L + (px - 1), (size_t)L * L);
        }
        asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    };
    // bounded wait for the commit; false (and the error word set) on timeout
    uint32_t phase = 0;
    const uint32_t bar = gen_smem_u32(&mbar);
    auto wait_mmas = [&]() -> bool {
        bool done = false;
        for (unsigned it = 0; it < kWaitLimit && !done; ++it) done = gen_mbar_try_wait(bar, phase);
        if (__syncthreads_or(!done)) {
            if (tid == 0) atomicExch(flag, 4);
            return false;
        }
        phase ^= 1u;
        return true;
    };

    const int first = blockIdx.x, stride = gridDim.x;
    const int n = (ntiles > first) ? (ntiles - first + stride - 1) / stride : 0;   // tiles of this CTA
    bool failed = false;
    for (int k = 0; k < n; ++k) {
        load_window(first + k * stride);
        asm volatile("cp.async.wait_all;" ::: "memory");
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        __syncthreads();
        if (tid == 0) issue_mmas();
        if (!wait_mmas()) {
            failed = true;
            break;
        }
        epilogue(first + k * stride);
        __syncthreads();
    }
    if (failed) {   // give in-flight MMAs a bounded chance to land before the TMEM is freed
        bool done = false;
        for (unsigned it = 0; it < kWaitLimit && !done; ++it) done = gen_mbar_try_wait(bar, phase);
    }
    asm volatile("cp.async.wait_all;" ::: "memory");
    __syncthreads();
    if (warp == 0)
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(kTmemCols) : "memory");
}

// TMA-fed variant for L = 128 (the configured size): a tile is one image row (128 positions =
// the 128 TMEM lanes). Its window is the three wrapped rows y-1, y, y+1, each staged as kCh
// blocks (one per 16-byte channel chunk) of 130 slots (x = -1 .. 128) by one TMA box
// [chunk elements, 130 x, 1 row, 1 chunk, 1 image] per block (a contiguous run of the chunk
// plane), completing on one mbarrier: 3 kCh bulk copies per tile. TMA fills x = -1 and x = 128 with
// zeros; the threads then copy x = 127 and x = 0 into those slots (periodic in x), fence them
// to the async proxy, and thread 0 issues the 9 taps x kCh/2 MMAs, each tap a descriptor offset
// (row block, and x shift of one slot). The next tile's copies are issued as soon as the MMAs
// have committed, so they land while the epilogue drains the accumulator.
namespace tma {
constexpr int kSlots = 130;                   // x = -1 .. 128
constexpr int kBlk = 2176;                    // bytes per (row, chunk) block: 130 x 16 B, 128-B aligned
// MMA N for co output channels: M = 128 takes N in multiples of 16
__host__ __device__ constexpr int nmma(int co) { return (co + 15) / 16 * 16; }
template <int MODE, int KCH, int CO>
__host__ __device__ constexpr int btap() { return (nmma(CO) / 8) * KCH * tc::kCore; }   // B bytes per tap
template <int MODE, int ICH = tc::chunks<MODE>(), int KCH = ICH, int CO = tc::kC, int R = 1>
__host__ __device__ constexpr int smem_bytes() { return 9 * btap<MODE, KCH, CO>() + (R + 2) * KCH * kBlk + 1024; }
}  // namespace tma

// Every convolution of the generator at L = 128 with TMA-staged windows. ICH input chunks
// (16 bytes of channels each) come in by TMA; the K of one tap is KCH chunks (KCH - ICH zero
// blocks when a layer's inputs do not fill an MMA's K: the first layer's 8 BF16 channels are
// one chunk of the two of K = 16); N = CO output channels rounded up to 16.
//   MODE 0: bias + ReLU, BF16 out (48 channels);  MODE 1: bias, FP32 out (48 channels);
//   MODE 2: TF32 data gradient, times (activation > 0), FP32 out;
//   MODE 3: bias, FP32 out of CO = 4 channels [pixel][4] (the generator's last layer).
// A tile is R consecutive output rows of one image: its window holds R + 2 input rows, the
// MMAs of output row j read window rows j .. j+2 into accumulator j (R x the TMEM columns),
// and one commit and one epilogue pass cover the R rows, so the per-tile latency of the copy,
// the commit and the epilogue is paid once for R rows.
// With wimg (the forward modes), the weights arrive by one bulk copy of their tensor-core image
// (k_gen_wimage) instead of being rearranged by the threads.
template <int MODE, int ICH, int KCH, int CO, int R>
__global__ void __launch_bounds__(128, 2)
k_gen_conv_tma(const __grid_constant__ CUtensorMap tmap, const __nv_bfloat16* __restrict__ w,
               const uint8_t* __restrict__ wimg, const float* __restrict__ bias,
               const __nv_bfloat16* __restrict__ mask, void* __restrict__ out_v, int ntiles,
               int* __restrict__ flag) {
    using namespace tc;
    using TA = typename Traits<MODE>::TA;
    constexpr int kEpc = Traits<MODE>::kEpc;
    constexpr int NN = tma::nmma(CO);
    constexpr int CI = ICH * kEpc;                           // real input channels
    constexpr int kBT = tma::btap<MODE, KCH, CO>();
    constexpr int kCols = NN <= 32 ? 32 : 64;                // TMEM columns of one accumulator
    constexpr int kL = kM;                                   // lattice edge of this kernel
    constexpr int kTpi = kL / R;                             // tiles per image
    constexpr uint32_t kTx = (R + 2u) * ICH * tma::kSlots * 16u;   // bytes per window (OOB fill included)
    static_assert(KCH % 2 == 0 && KCH >= ICH && NN <= 64 && (MODE != 3 || CO == 4) && (MODE == 3 || CO == kC) &&
                  (R == 1 || R == 2 || R == 4) && kL % R == 0, "convolution shape");
    extern __shared__ uint8_t tsm_raw[];
    __shared__ __align__(8) unsigned long long mbar;       // MMA commit
    __shared__ __align__(8) unsigned long long tbar;       // window copies
    __shared__ __align__(8) unsigned long long wbar;       // weight image copy
    __shared__ uint32_t tmem_slot;
    __shared__ __align__(16) float sbias[NN];
    uint8_t* sB = (uint8_t*)(((uintptr_t)tsm_raw + 1023) & ~(uintptr_t)1023);
    uint8_t* sA = sB + 9 * kBT;                             // 1024-aligned + 9 kBT (multiple of 128)
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;

    const uint32_t aBase = gen_smem_u32(sA), bBase = gen_smem_u32(sB);
    const uint32_t mb = gen_smem_u32(&mbar), tb = gen_smem_u32(&tbar), wbr = gen_smem_u32(&wbar);
    const bool use_img = MODE != 2 && wimg != nullptr;
    // thread 0: the window of tile t (image t / kTpi, rows R (t % kTpi) ..): R + 2 rows x ICH chunk blocks
    auto issue_window = [&](int t) {
        const int img = t / kTpi, y = (t - img * kTpi) * R;
        asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(tb), "r"(kTx) : "memory");
#pragma unroll
        for (int r = 0; r < R + 2; ++r) {
            int yy = y + r - 1;
            yy += (yy < 0) ? kL : ((yy >= kL) ? -kL : 0);
#pragma unroll
            for (int c = 0; c < ICH; ++c) {
                const uint32_t dst = aBase + (uint32_t)((r * KCH + c) * tma::kBlk);
                asm volatile(
                    "cp.async.bulk.tensor.5d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4, "
                    "%5, %6}], [%7];" ::"r"(dst),
                    "l"(reinterpret_cast<uint64_t>(&tmap)), "r"(0), "r"(-1), "r"(yy), "r"(c), "r"(img), "r"(tb)
                    : "memory");
            }
        }
    };
    const int first = blockIdx.x, stride = gridDim.x;
    const int n = (ntiles > first) ? (ntiles - first + stride - 1) / stride : 0;
    if (tid == 0) {
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(mb) : "memory");
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(tb) : "memory");
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(wbr) : "memory");
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        if (n > 0) issue_window(first);   // the first window lands while the weights are staged
        if (use_img && n > 0) {
            asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(wbr), "r"(9u * kBT) : "memory");
            asm volatile(
                "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(bBase),
                "l"(reinterpret_cast<uint64_t>(wimg)), "r"(9u * kBT), "r"(wbr)
                : "memory");
        }
    }
    if constexpr (KCH > ICH) {   // K-padding blocks: zero once, never written by TMA
        constexpr int kZ = KCH - ICH, kU = tma::kBlk / 16;
        for (int i = tid; i < (R + 2) * kZ * kU; i += blockDim.x) {
            const int zb = i / kU, r = zb / kZ, c = ICH + (zb - r * kZ);
            *(uint4*)(sA + (r * KCH + c) * tma::kBlk + (i - zb * kU) * 16) = make_uint4(0, 0, 0, 0);
        }
    }
    if (use_img) {
        // weights by the bulk copy above
    } else if constexpr (ICH == KCH && CI == kC && CO == kC) {
        stage_weights<MODE>(sB, w, tid, blockDim.x);   // 48 -> 48: 16-byte loads
    } else {
        // w[tap][k][n] (CI x CO) -> B_tap[n][k] over the padded NN x KCH*epc, zeros outside
        constexpr int KK = KCH * kEpc;
#pragma unroll 8
        for (int i = tid; i < 9 * NN * KK; i += blockDim.x) {
            const int tap = i / (NN * KK), r = i - tap * NN * KK, nn = r / KK, k = r - nn * KK;
            const float v = (nn < CO && k < CI) ? __bfloat162float(__ldg(w + (tap * CI + k) * CO + nn)) : 0.0f;
            *(TA*)(sB + tap * kBT + ((nn >> 3) * KCH + k / kEpc) * kCore + (nn & 7) * 16 + (k % kEpc) * (int)sizeof(TA)) =
                (TA)v;
        }
    }
    if (tid < NN) sbias[tid] = (MODE == 2 || tid >= CO) ? 0.0f : bias[tid];
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(gen_smem_u32(&tmem_slot)),
                     "r"(R * kCols)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const uint32_t tmem = tmem_slot;
    uint32_t mphase = 0, tphase = 0;
    auto bounded_wait = [&](uint32_t bar, uint32_t& ph, int code) -> bool {
        bool done = false;
        for (unsigned it = 0; it < kWaitLimit && !done; ++it) done = gen_mbar_try_wait(bar, ph);
        if (__syncthreads_or(!done)) {
            if (tid == 0) atomicExch(flag, code);
            return false;
        }
        ph ^= 1u;
        return true;
    };

    bool failed = false, window_pending = n > 0, weights_pending = use_img && n > 0;
    if (weights_pending) {
        uint32_t wph = 0;
        if (!bounded_wait(wbr, wph, 6)) failed = true;
        else weights_pending = false;
    }
    for (int k = 0; k < n && !failed; ++k) {
        const int t = first + k * stride;
        if (!bounded_wait(tb, tphase, 5)) {
            failed = true;
            break;
        }
        window_pending = false;
        // periodic x: slot 0 <- x = 127 (slot 128), slot 129 <- x = 0 (slot 1), in the loaded blocks
        if (tid < (R + 2) * ICH * 2) {
            const int e = tid >> 1, r = e / ICH, c = e - r * ICH;
            uint8_t* blk = sA + (r * KCH + c) * tma::kBlk;
            const int to = (tid & 1) ? (tma::kSlots - 1) : 0, from = (tid & 1) ? 1 : kL;
            *(uint4*)(blk + to * 16) = *(const uint4*)(blk + from * 16);
        }
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
        __syncthreads();
        if (tid == 0) {
            asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
#pragma unroll
            for (int j = 0; j < R; ++j) {
#pragma unroll 1
                for (int tap = 0; tap < 9; ++tap) {
                    const int ty = tap / 3, tx = tap - 3 * ty;
#pragma unroll
                    for (int ks = 0; ks < KCH / 2; ++ks) {
                        const uint64_t ad = umma_desc(aBase + (uint32_t)(((j + ty) * KCH + 2 * ks) * tma::kBlk + tx * 16),
                                                      (uint32_t)tma::kBlk, 128);
                        const uint64_t bd = umma_desc(bBase + tap * kBT + 2 * ks * kCore, kCore, KCH * kCore);
                        tc_mma<MODE, NN>(tmem + (uint32_t)(j * kCols), ad, bd, (tap | ks) ? 1u : 0u);
                    }
                }
            }
            asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(mb)
                         : "memory");
        }
        if (!bounded_wait(mb, mphase, 4)) {
            failed = true;
            break;
        }
        // the MMAs have read the window: the next tile's copies overlap this epilogue
        if (k + 1 < n) {
            if (tid == 0) issue_window(t + stride);
            window_pending = true;
        }
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        const int img = t / kTpi, y0 = (t - img * kTpi) * R;
#pragma unroll 1
        for (int jr = 0; jr < R; ++jr) {
            float v[NN];
            const uint32_t taddr = tmem + (uint32_t)(jr * kCols) + ((uint32_t)(warp * 32) << 16);
#pragma unroll
            for (int j = 0; j < NN / 16; ++j) tmem_ld16(taddr + 16 * j, v + 16 * j);
            asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
            const size_t pp = (size_t)(y0 + jr) * kL + (size_t)(warp * 32 + lane);
            if constexpr (MODE == 3) {
                float4* dst = reinterpret_cast<float4*>(out_v) + (size_t)img * kL * kL + pp;
                *dst = make_float4(v[0] + sbias[0], v[1] + sbias[1], v[2] + sbias[2], v[3] + sbias[3]);
            } else {
                conv_store<MODE>(v, sbias, out_v, mask, (size_t)img, pp, (size_t)kL * kL);
            }
        }
        asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    }
    if (failed) {   // bounded waits for what may still be in flight before the TMEM is freed
        bool done = false;
        for (unsigned it = 0; it < kWaitLimit && !done; ++it) done = gen_mbar_try_wait(mb, mphase);
    }
    if (window_pending) {
        bool done = false;
        for (unsigned it = 0; it < kWaitLimit && !done; ++it) done = gen_mbar_try_wait(tb, tphase);
    }
    if (weights_pending) {
        bool done = false;
        for (unsigned it = 0; it < kWaitLimit && !done; ++it) done = gen_mbar_try_wait(wbr, 0);
    }
    __syncthreads();
    if (warp == 0)
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(R * kCols) : "memory");
}

// TMA-fed, warp-specialised forward convolution for L = 128 (BF16 modes), opt-in: one CTA per
// SM, a ring of kWsStages windows and two TMEM accumulators, so the copies of later tiles, the
// MMAs of tile k and the epilogue of tile k-1 overlap. Measured on GB300 (16 x 128^2, chunk-
// planar activations) a warm-start pass takes 0.379 ms with it against 0.358 ms with two
// single-role TMA CTAs per SM, which overlap one another's phases.
//   warps 0-3: epilogue (warp w drains TMEM lanes 32w ..), then arrive on tempty[acc];
//   warp 4:    producer (lane 0): after empty[stage], expect_tx on full[stage] and the
//              window's 3 x kCh blocks, each one box of 130 slots (x = -1 .. 128, the two
//              edge slots zero-filled) into a 128-byte aligned block;
//   warp 5:    MMA issue: after full[stage] the 32 lanes copy the wrapped edge columns
//              (x = 127 into slot 0, x = 0 into slot 129) and fence them to the async proxy;
//              after tempty[acc] lane 0 issues the 27 MMAs and commits them to empty[stage]
//              and tfull[acc]; the warp owns the TMEM allocation.
// Every wait is bounded; a role that gives up sets the error word and stops, and the others
// then time out on the barriers it no longer signals.
constexpr int kWsStages = 4;
constexpr int kTwsThreads = 192;
template <int MODE>
__host__ __device__ constexpr int tmaws_smem_bytes() {
    return 9 * tc::btap<MODE>() + kWsStages * 3 * tc::chunks<MODE>() * tma::kBlk + 1024;
}

template <int MODE>
__global__ void __launch_bounds__(kTwsThreads, 1)
k_gen_conv_tmaws(const __grid_constant__ CUtensorMap tmap, const __nv_bfloat16* __restrict__ w, const float* __restrict__ bias, void* __restrict__ out_v,
                 int ntiles, int* __restrict__ flag) {
    static_assert(MODE == 0 || MODE == 1, "BF16 modes only");
    using namespace tc;
    constexpr int kCh = chunks<MODE>();
    constexpr int kBT = btap<MODE>();
    constexpr int kL = kM;
    constexpr int kS = kWsStages;
    constexpr uint32_t kWin = 3u * kCh * tma::kBlk;                // bytes per ring stage
    constexpr uint32_t kTx = 3u * kCh * tma::kSlots * 16u;         // bytes per window
    extern __shared__ uint8_t tsm_raw[];
    __shared__ __align__(8) unsigned long long bars[2 * kS + 4];   // full[S], empty[S], tfull[2], tempty[2]
    __shared__ uint32_t tmem_slot;
    __shared__ __align__(16) float sbias[kC];
    uint8_t* sB = (uint8_t*)(((uintptr_t)tsm_raw + 1023) & ~(uintptr_t)1023);
    uint8_t* sA = sB + 9 * kBT;
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;

    if (warp == 5) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(gen_smem_u32(&tmem_slot)),
                     "r"(2 * kTmemCols)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    if (tid == 0) {
        for (int b = 0; b < 2 * kS + 4; ++b) {
            const unsigned cnt = (b >= 2 * kS + 2) ? 128u : 1u;
            asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(gen_smem_u32(&bars[b])), "r"(cnt) : "memory");
        }
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const uint32_t tmem = tmem_slot;
    const uint32_t aBase = gen_smem_u32(sA), bBase = gen_smem_u32(sB);
    const uint32_t full0 = gen_smem_u32(&bars[0]), empty0 = gen_smem_u32(&bars[kS]);
    const uint32_t tfull0 = gen_smem_u32(&bars[2 * kS]), tempty0 = gen_smem_u32(&bars[2 * kS + 2]);
    const int first = blockIdx.x, stride = gridDim.x;
    const int n = (ntiles > first) ? (ntiles - first + stride - 1) / stride : 0;
    auto wait = [&](uint32_t bar, uint32_t parity) -> bool {
        for (unsigned it = 0; it < kWaitLimit; ++it)
            if (gen_mbar_try_wait(bar, parity)) return true;
        atomicExch(flag, 6);
        return false;
    };
    auto tma_box = [&](uint32_t dst, int c, int y, int img, uint32_t bar) {   // x = -1 .. 128
        asm volatile(
            "cp.async.bulk.tensor.5d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4, %5, "
            "%6}], [%7];" ::"r"(dst),
            "l"(reinterpret_cast<uint64_t>(&tmap)), "r"(0), "r"(-1), "r"(y), "r"(c), "r"(img), "r"(bar)
            : "memory");
    };
    // producer: the window of the CTA's tile k into stage k % S
    auto issue = [&](int k) {
        const int t = first + k * stride, img = t / kL, y = t - img * kL, st = k % kS;
        const uint32_t bar = full0 + 8 * st;
        asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(kTx) : "memory");
#pragma unroll 1
        for (int r = 0; r < 3; ++r) {
            int yy = y + r - 1;
            yy += (yy < 0) ? kL : ((yy >= kL) ? -kL : 0);
#pragma unroll 1
            for (int c = 0; c < kCh; ++c) {
                tma_box(aBase + (uint32_t)st * kWin + (uint32_t)((r * kCh + c) * tma::kBlk), c, yy, img, bar);
            }
        }
    };
    // the first stages are in flight while the weights are staged
    if (warp == 4 && lane == 0)
        for (int k = 0; k < n && k < kS; ++k) issue(k);
    stage_weights<MODE>(sB, w, tid, blockDim.x);
    if (tid < kC) sbias[tid] = bias[tid];
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    __syncthreads();

    if (warp == 4) {
        // ---- producer ----
        if (lane == 0) {
            int issued = (n < kS) ? n : kS;
            for (int k = kS; k < n; ++k) {
                if (!wait(empty0 + 8 * (k % kS), ((k / kS) - 1) & 1)) break;   // MMAs of tile k - S done
                issue(k);
                issued = k + 1;
            }
            // nothing of ours may land after the CTA ends: the last use of every stage completes
            for (int j = (issued > kS ? issued - kS : 0); j < issued; ++j) wait(full0 + 8 * (j % kS), (j / kS) & 1);
        }
        __syncwarp();
    } else if (warp == 5) {
        // ---- edge columns and MMA issue ----
        int k = 0;
        for (; k < n; ++k) {
            const int st = k % kS, ac = k & 1;
            if (!__all_sync(0xffffffffu, wait(full0 + 8 * st, (k / kS) & 1))) break;
            // periodic x: slot 0 <- x = 127 (slot 128), slot 129 <- x = 0 (slot 1); 3 kCh blocks
            for (int e = lane; e < 3 * kCh * 2; e += 32) {
                uint8_t* blk = sA + st * kWin + (e >> 1) * tma::kBlk;
                const int to = (e & 1) ? (tma::kSlots - 1) : 0, from = (e & 1) ? 1 : kL;
                *(uint4*)(blk + to * 16) = *(const uint4*)(blk + from * 16);
            }
            asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
            __syncwarp();
            bool go = true;
            if (lane == 0) {
                if (k >= 2 && !wait(tempty0 + 8 * ac, ((k >> 1) - 1) & 1)) go = false;
            }
            if (!__shfl_sync(0xffffffffu, go, 0)) break;
            if (lane == 0) {
                asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
                const uint32_t a0 = aBase + (uint32_t)st * kWin, d = tmem + (uint32_t)(ac * kTmemCols);
#pragma unroll 1
                for (int tap = 0; tap < 9; ++tap) {
                    const int ty = tap / 3, tx = tap - 3 * ty;
#pragma unroll
                    for (int ks = 0; ks < kCh / 2; ++ks) {
                        const uint64_t ad = umma_desc(a0 + (uint32_t)((ty * kCh + 2 * ks) * tma::kBlk + tx * 16),
                                                      (uint32_t)tma::kBlk, 128);
                        const uint64_t bd = umma_desc(bBase + tap * kBT + 2 * ks * kCore, kCore, kCh * kCore);
                        tc_mma<MODE>(d, ad, bd, (tap | ks) ? 1u : 0u);
                    }
                }
                asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                                 empty0 + 8 * st)
                             : "memory");
                asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                                 tfull0 + 8 * ac)
                             : "memory");
            }
            __syncwarp();
        }
        // the TMEM is freed only after the last committed MMAs have landed
        if (lane == 0 && k > 0) wait(tfull0 + 8 * ((k - 1) & 1), ((k - 1) >> 1) & 1);
        __syncwarp();
    } else {
        // ---- epilogue (warps 0-3) ----
        for (int k = 0; k < n; ++k) {
            const int ac = k & 1;
            if (!wait(tfull0 + 8 * ac, (k >> 1) & 1)) break;
            asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
            const int t = first + k * stride, img = t / kL, y = t - img * kL;
            float v[kC];
            const uint32_t taddr = tmem + (uint32_t)(ac * kTmemCols) + ((uint32_t)(warp * 32) << 16);
            tmem_ld16(taddr + 0, v);
            tmem_ld16(taddr + 16, v + 16);
            tmem_ld16(taddr + 32, v + 32);
            asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
            asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
            asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(tempty0 + 8 * ac) : "memory");
            conv_store<MODE>(v, sbias, out_v, nullptr, (size_t)img, (size_t)y * kL + (size_t)(warp * 32 + lane), (size_t)kL * kL);
        }
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    if (warp == 5)
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(2 * kTmemCols) : "memory");
}

// Warp-specialised variant of the BF16 modes (forward and probe), opt-in: one CTA per SM with a
// two-stage window ring and two TMEM accumulators, so the loads of tile k+1, the MMAs of tile k
// and the epilogue of tile k-1 run at once. Measured on GB300 at 16 x 128^2 it is slower than
// two single-role CTAs per SM (75.7 vs 61.6 us per layer): the two producer warps and their
// cp.async completion waits (long-scoreboard stalls) bound the tile rate, not the MMAs.
//   warps 0-3: epilogue (warp w drains TMEM lanes 32w ..), then arrive on tempty[acc];
//   warps 4-5: producers: cp.async of tile k into ring slot k&1 (after empty[slot]), one
//              commit group per tile; once the previous tile's group has landed, fence it to
//              the async proxy and arrive on full[slot];
//   warp 6:    MMA issue (lane 0): wait full[slot] and tempty[acc], 27 MMAs, commit to
//              empty[slot] and tfull[acc]; the warp owns the TMEM allocation.
// Every wait is bounded; a role that gives up sets the error word and stops, and the others
// then time out on the barriers it no longer signals.
constexpr int kWsThreads = 224;

template <int MODE>
__host__ __device__ constexpr int ws_smem_bytes(int L) {
    return 9 * tc::btap<MODE>() + 2 * tc::chunks<MODE>() * tc::window(L) * 16 + 1024;
}

template <int MODE>
__global__ void __launch_bounds__(kWsThreads, 1)
k_gen_conv_ws(const __nv_bfloat16* __restrict__ in, const __nv_bfloat16* __restrict__ w,
              const float* __restrict__ bias, void* __restrict__ out_v, int L, int tiles_per_img, int ntiles,
              int* __restrict__ flag) {
    static_assert(MODE == 0 || MODE == 1, "BF16 modes only");
    using namespace tc;
    constexpr int kCh = chunks<MODE>();        // 6
    constexpr int kBT = btap<MODE>();
    constexpr int kProd = 64;                  // producer threads
    constexpr int kRound = 10;                 // window positions per producer round (60 threads)
    extern __shared__ uint8_t tsm_raw[];
    __shared__ __align__(8) unsigned long long bars[8];   // full[2], empty[2], tfull[2], tempty[2]
    __shared__ uint32_t tmem_slot;
    __shared__ __align__(16) float sbias[kC];
    uint8_t* sB = (uint8_t*)(((uintptr_t)tsm_raw + 1023) & ~(uintptr_t)1023);
    uint8_t* sA = sB + 9 * kBT;
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int P = L + 2, W = window(L), npad = P * P;
    const uint32_t winBytes = (uint32_t)(kCh * W * 16);

    stage_weights<MODE>(sB, w, tid, blockDim.x);
    if (tid < kC) sbias[tid] = bias[tid];
    if (warp == 6) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(gen_smem_u32(&tmem_slot)),
                     "r"(2 * kTmemCols)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    if (tid == 0) {
        const unsigned counts[8] = {kProd, kProd, 1, 1, 1, 1, 128, 128};
        for (int b = 0; b < 8; ++b)
            asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(gen_smem_u32(&bars[b])), "r"(counts[b]) : "memory");
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const uint32_t tmem = tmem_slot;
    const uint32_t aBase = gen_smem_u32(sA), bBase = gen_smem_u32(sB);
    const uint32_t full0 = gen_smem_u32(&bars[0]), empty0 = gen_smem_u32(&bars[2]);
    const uint32_t tfull0 = gen_smem_u32(&bars[4]), tempty0 = gen_smem_u32(&bars[6]);
    const int first = blockIdx.x, stride = gridDim.x;
    const int n = (ntiles > first) ? (ntiles - first + stride - 1) / stride : 0;
    auto wait = [&](uint32_t bar, uint32_t parity) -> bool {
        for (unsigned it = 0; it < (1u << 24); ++it)   // bounded polls
            if (gen_mbar_try_wait(bar, parity)) return true;
        atomicExch(flag, 4);
        return false;
    };
    auto arrive = [&](uint32_t bar) {
        asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(bar) : "memory");
    };

    if (warp >= 4 && warp < 6) {
        // ---- producers ----
        const int pt = tid - 128;
        auto issue = [&](int k) {
            const int t = first + k * stride, img = t / tiles_per_img;
            const int w0 = (t - img * tiles_per_img) * kM - 1;
            const __nv_bfloat16* src_img = in + (size_t)img * L * L * kC;
            if (pt < kRound * kCh) {
                const int c = pt % kCh;
                int j = pt / kCh, pos = w0 + j;
                int py = (pos >= 0) ? pos / P : -1;
                int px = pos - py * P;
                const uint32_t dst0 = aBase + (uint32_t)(k & 1) * winBytes + (uint32_t)(c * W * 16);
                for (; j < W; j += kRound, pos += kRound) {
                    const bool inside = pos >= 0 && pos < npad;
                    const uint4* src = (const uint4*)src_img;
                    if (inside) {
                        int y = py - 1, x = px - 1;
                        y += (y < 0) ? L : ((y >= L) ? -L : 0);
                        x += (x < 0) ? L : ((x >= L) ? -L : 0);
                        src = (const uint4*)src_img + ((size_t)c * L * L + (size_t)y * L + x);   // chunk plane c
                    }
                    asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;" ::"r"(dst0 + (uint32_t)(j * 16)),
                                 "l"(src), "r"(inside ? 16 : 0)
                                 : "memory");
                    px += kRound;
                    if (px >= P) {
                        px -= P;
                        ++py;
                    }
                }
            }
            asm volatile("cp.async.commit_group;" ::: "memory");
        };
        bool ok = true;
        for (int k = 0; k < n && ok; ++k) {
            if (k >= 2) ok = wait(empty0 + 8 * (k & 1), ((k >> 1) - 1) & 1);   // MMAs of tile k-2 done
            if (!ok) break;
            issue(k);
            if (k >= 1) {   // tile k-1 landed: publish it
                asm volatile("cp.async.wait_group 1;" ::: "memory");
                asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
                arrive(full0 + 8 * ((k - 1) & 1));
            }
        }
        asm volatile("cp.async.wait_group 0;" ::: "memory");
        if (ok && n > 0) {
            asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
            arrive(full0 + 8 * ((n - 1) & 1));
        }
    } else if (warp == 6) {
        // ---- MMA issue ----
        if (lane == 0) {
            for (int k = 0; k < n; ++k) {
                const int sl = k & 1;
                if (!wait(full0 + 8 * sl, (k >> 1) & 1)) break;
                if (k >= 2 && !wait(tempty0 + 8 * sl, ((k >> 1) - 1) & 1)) break;
                asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
                const uint32_t a0 = aBase + (uint32_t)sl * winBytes, d = tmem + (uint32_t)(sl * kTmemCols);
#pragma unroll 1
                for (int tap = 0; tap < 9; ++tap) {
                    const int shift = (P + 1) + (tap / 3 - 1) * P + (tap % 3 - 1);
#pragma unroll
                    for (int ks = 0; ks < kCh / 2; ++ks) {
                        const uint64_t ad =
                            umma_desc(a0 + (uint32_t)((2 * ks * W + shift) * 16), (uint32_t)(W * 16), 128);
                        const uint64_t bd = umma_desc(bBase + tap * kBT + 2 * ks * kCore, kCore, kCh * kCore);
                        tc_mma<MODE>(d, ad, bd, (tap | ks) ? 1u : 0u);
                    }
                }
                asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                                 empty0 + 8 * sl)
                             : "memory");
                asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                                 tfull0 + 8 * sl)
                             : "memory");
            }
        }
        __syncwarp();
    } else {
        // ---- epilogue (warps 0-3) ----
        for (int k = 0; k < n; ++k) {
            const int ac = k & 1;
            if (!wait(tfull0 + 8 * ac, (k >> 1) & 1)) break;
            asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
            const int t = first + k * stride, img = t / tiles_per_img;
            const int q0 = P + (t - img * tiles_per_img) * kM;
            float v[kC];
            const uint32_t taddr = tmem + (uint32_t)(ac * kTmemCols) + ((uint32_t)(warp * 32) << 16);
            tmem_ld16(taddr + 0, v);
            tmem_ld16(taddr + 16, v + 16);
            tmem_ld16(taddr + 32, v + 32);
            asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
            asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
            arrive(tempty0 + 8 * ac);   // the accumulator may be overwritten now
            const int pos = q0 + warp * 32 + lane, py = pos / P, px = pos - py * P;
            if (py >= 1 && py <= L && px >= 1 && px <= L) {
                conv_store<MODE>(v, sbias, out_v, nullptr, (size_t)img, (size_t)(py - 1) * L + (px - 1), (size_t)L * L);
            }
        }
    }
    // every committed MMA has been drained by the epilogue (or timed out); free the TMEM
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    if (warp == 6)
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(2 * kTmemCols) : "memory");
}

// ------------------------------------------------------------------------------------------
// Weight gradient of a hidden layer on the tensor cores: dW[tap][ci][co] = sum_p
// in[p + tap, ci] * dout[p, co], the positions p as the contraction (kind::f16, FP32
// accumulators in tensor memory). The layer input is BF16 already; the FP32 output gradient
// is split into BF16 hi + lo (lo = the remainder rounded again, 16 significant bits in all)
// and both halves are multiplied into the same accumulator, which is more accurate than TF32.
// A K-block is W = min(L, 64) consecutive positions of one image row. Both operands are
// MN-major: a slot holds 8 channels (16 bytes) per position, the positions 16 bytes apart, so
// the window of a tap shifted by dx positions is the same slot started dx * 16 bytes later
// and the layer input is staged once per K-block (rows y-1, y, y+1 and columns x0-1 .. x0+W,
// periodic), not once per tap. A row block holds 8 slots (6 of data, 2 of zeros) = 64 rows,
// so one M = 128 MMA covers two vertical taps: for each dx, tile P starts at row block 0 (its
// rows 0-63 are tap (-1, dx), rows 64-127 tap (0, dx)) and tile Q at row block 1 (rows 64-127
// tap (+1, dx); its first half repeats P's second and is not read). B is the output gradient
// (6 slots, N = 48). Six accumulators of 48 columns.
// Warp-specialised over a ring of kStages slots (mbarriers loaded / full / empty per slot):
//   warp 0:          producer: after `empty` (the slot's previous MMAs completed), lane 0 sets
//                    the byte count of `loaded` (expect_tx) and 30 lanes issue bulk copies of
//                    the K-block's input rows (one lane per row and channel group, in runs
//                    split at the periodic x edge) and raw FP32 gradient rows (one lane each);
//   warp 1, lane 0:  MMA issuer: after `full`, 6 tiles x W/16 steps x (hi, lo) MMAs, committed
//                    to `empty`;
//   warps 2-15:      after `loaded`, convert the raw gradient to the hi / lo operands in the
//                    slot and arrive on `full` (one arrival per warp).
// Every wait is bounded and also ends when another role gave up (a shared abort word); the
// producer lets its last copies land and the epilogue waits for the last commit before the
// tensor memory is freed. Each CTA covers a strided set of K-blocks over the batch; its
// partial dW (read back with tcgen05.ld) goes to `part` and k_gen_sum_parts adds the partials
// in a fixed order.
// ------------------------------------------------------------------------------------------
namespace wg {
constexpr int kWMax = 64;                                 // positions per K-block at most
constexpr int kSlotA = (kWMax + 2) * 16;                  // bytes per input slot (with the halo)
constexpr int kSlot = kWMax * 16;                         // bytes per gradient slot (raw or BF16)
constexpr int kBytesA = 3 * 8 * kSlotA;                   // 25344: 3 row blocks x 8 slots
constexpr int kBytesR = tc::kC / 4 * kSlot;               // 12288: raw FP32 gradient, 12 slots
constexpr int kBytesB = tc::kC / 8 * kSlot;               // 6144: BF16 gradient, 6 slots (hi or lo)
constexpr int kStages = 4;
constexpr int kStage = kBytesA + kBytesR + 2 * kBytesB;   // 49920: one ring slot
constexpr int kThreads = 512;
constexpr int kConvWarps = kThreads / 32 - 2;
constexpr int kCols = 512;                                // six accumulators at 64-column steps
constexpr size_t kSmem = (size_t)kStages * kStage + 1024;
// BF16 A and B, both MN-major (instruction-descriptor bits 15 and 16), N = 48, M = 128
constexpr uint32_t kIdesc = tc::idesc<0, tc::kC>() | (1u << 15) | (1u << 16);
// K-block length for an L x L image (0: the tensor-core form does not apply)
__host__ __device__ constexpr int block_len(int L) {
    return (L % 16 != 0) ? 0 : (L <= kWMax ? L : (L % kWMax == 0 ? kWMax : 0));
}
__device__ __forceinline__ void mma(uint32_t tmem, uint64_t ad, uint64_t bd, uint32_t acc) {
    asm volatile(
        "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(tmem),
        "l"(ad), "l"(bd), "r"(kIdesc), "r"(acc)
        : "memory");
}
__device__ __forceinline__ void bulk(uint32_t dst, const void* src, uint32_t bytes, uint32_t bar) {
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(dst),
                 "l"(src), "r"(bytes), "r"(bar)
                 : "memory");
}
__device__ __forceinline__ uint32_t pack_bf16(float a, float b) {
    const __nv_bfloat162 h = __floats2bfloat162_rn(a, b);
    return *reinterpret_cast<const uint32_t*>(&h);
}
// bounded wait for phase `parity` of `bar`; gives up (abort word and error flag set) after
// `limit` polls or as soon as another role has given up
__device__ __forceinline__ bool wait(uint32_t bar, uint32_t parity, volatile int* abort, int* flag) {
    for (unsigned it = 0; it < tc::kWaitLimit; ++it) {
        if (gen_mbar_try_wait(bar, parity)) return true;
        if (*abort) return false;
    }
    *abort = 1;
    atomicExch(flag, 4);
    return false;
}
}  // namespace wg

template <int KS>   // MMA K-steps (16 positions) per K-block: W = 16 KS
__global__ void __launch_bounds__(wg::kThreads, 1)
k_gen_wgrad_tc(const __nv_bfloat16* __restrict__ in, const float* __restrict__ dout, float* __restrict__ part,
               int L, int nkb, int* __restrict__ flag) {
    using namespace wg;
    constexpr int kC = tc::kC, W = 16 * KS;
    extern __shared__ uint8_t wsm_raw[];
    __shared__ __align__(8) unsigned long long loaded[kStages], full[kStages], empty[kStages];
    __shared__ uint32_t tmem_slot;
    __shared__ int last_mma;
    __shared__ volatile int abort_word;
    uint8_t* smem = (uint8_t*)(((uintptr_t)wsm_raw + 1023) & ~(uintptr_t)1023);
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const size_t LL = (size_t)L * L;
    const int bpr = L / W;                                  // K-blocks per image row
    const uint32_t sbase = gen_smem_u32(smem);
    const int first = blockIdx.x, stride = gridDim.x;
    const int n = (nkb > first) ? (nkb - first + stride - 1) / stride : 0;

    // the zero slots 6 and 7 of each row block, in every ring slot (never copied over)
    for (int i = tid; i < kStages * 3 * 2 * (kSlotA / 16); i += kThreads) {
        const int c = i % (kSlotA / 16), s = i / (kSlotA / 16);
        const int st = s / 6, slot = (s % 6) / 2 * 8 + 6 + s % 2;
        *reinterpret_cast<uint4*>(smem + st * kStage + slot * kSlotA + c * 16) = make_uint4(0, 0, 0, 0);
    }
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(gen_smem_u32(&tmem_slot)),
                     "r"(kCols)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    if (tid == 0) {
        for (int s = 0; s < kStages; ++s) {
            asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(gen_smem_u32(&loaded[s])) : "memory");
            asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(gen_smem_u32(&full[s])), "r"(kConvWarps)
                         : "memory");
            asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(gen_smem_u32(&empty[s])) : "memory");
        }
        abort_word = 0;
        last_mma = -1;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    // the zeroed slots are read by the tensor cores (async proxy)
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const uint32_t tmem = tmem_slot;
    auto par = [](int j) { return (uint32_t)(j / kStages) & 1u; };

    if (warp == 0) {   // producer: lane 0 waits and sets the byte count, lanes 0-29 copy
        constexpr uint32_t kTx = 3u * (kC / 8) * (W + 2) * 16 + (kC / 4) * W * 16;
        int hi_fill = -1;
        for (int j = 0; j < n; ++j) {
            const int s = j % kStages;
            if (j >= kStages) {
                const bool ok = lane == 0 ? wait(gen_smem_u32(&empty[s]), par(j - kStages), &abort_word, flag) : true;
                if (!__shfl_sync(0xFFFFFFFFu, ok, 0)) break;
                asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
            }
            const int kb = first + j * stride;
            const int img = kb / (L * bpr), rem = kb - img * (L * bpr);
            const int y = rem / bpr, x0 = (rem - y * bpr) * W;
            const uint32_t bar = gen_smem_u32(&loaded[s]);
            const uint32_t sA = sbase + (uint32_t)(s * kStage), sR = sA + (uint32_t)kBytesA;
            if (lane == 0)
                asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(kTx) : "memory");
            __syncwarp();
            if (lane < 3 * (kC / 8)) {   // input rows y-1, y, y+1 of channel group h
                const int R = lane / (kC / 8), h = lane - R * (kC / 8);
                const int yy = (y + R - 1 + L) % L;
                const __nv_bfloat16* row = in + (((size_t)img * (kC / 8) + h) * LL + (size_t)yy * L) * 8;
                const uint32_t dst = sA + (uint32_t)((R * 8 + h) * kSlotA);
                int c = 0;
                while (c < W + 2) {   // runs of columns x0-1 .. x0+W, split at the periodic edge
                    const int x = (x0 - 1 + c + L) % L;
                    const int run = min(W + 2 - c, L - x);
                    bulk(dst + (uint32_t)(c * 16), row + (size_t)x * 8, (uint32_t)run * 16, bar);
                    c += run;
                }
            } else if (lane < 3 * (kC / 8) + kC / 4) {   // gradient slot g (4 channels)
                const int g = lane - 3 * (kC / 8);
                bulk(sR + (uint32_t)(g * kSlot), dout + (((size_t)img * (kC / 4) + g) * LL + (size_t)y * L + x0) * 4,
                     (uint32_t)W * 16, bar);
            }
            hi_fill = j;
        }
        // the last fill of every slot lands before the CTA's shared memory can be released
        if (lane == 0)
            for (int j = max(0, hi_fill - kStages + 1); j <= hi_fill; ++j)
                for (unsigned it = 0; it < (tc::kWaitLimit >> 4); ++it)
                    if (gen_mbar_try_wait(gen_smem_u32(&loaded[j % kStages]), par(j))) break;
    } else if (warp == 1) {
        if (lane == 0) {   // MMA issuer
            for (int k = 0; k < n; ++k) {
                const int s = k % kStages;
                if (!wait(gen_smem_u32(&loaded[s]), par(k), &abort_word, flag) ||
                    !wait(gen_smem_u32(&full[s]), par(k), &abort_word, flag))
                    break;
                asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
                // MN-major, no swizzle: LBO = 128 (8-position K groups), SBO = one slot (8-channel
                // MN groups); the start address field (bits 0-13, address >> 4) is offset per MMA
                const uint32_t sA = sbase + (uint32_t)(s * kStage);
                const uint64_t a0 = umma_desc(sA, 128, kSlotA);
                const uint64_t b0 = umma_desc(sA + (uint32_t)(kBytesA + kBytesR), 128, kSlot);
#pragma unroll
                for (int t = 0; t < 6; ++t) {
                    const int dxi = t >> 1, pq = t & 1;
#pragma unroll
                    for (int ks = 0; ks < KS; ++ks) {
                        const uint64_t ad = a0 + (uint64_t)((pq * 8 * kSlotA + (dxi + 16 * ks) * 16) >> 4);
                        mma(tmem + (uint32_t)(t * 64), ad, b0 + (uint64_t)((ks * 256) >> 4), (k | ks) ? 1u : 0u);
                        mma(tmem + (uint32_t)(t * 64), ad, b0 + (uint64_t)((kBytesB + ks * 256) >> 4), 1u);
                    }
                }
                asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                                 gen_smem_u32(&empty[s]))
                             : "memory");
                last_mma = k;
            }
        }
    } else {   // converters
        const int ct = tid - 64;
        for (int j = 0; j < n; ++j) {
            const int s = j % kStages;
            if (!wait(gen_smem_u32(&loaded[s]), par(j), &abort_word, flag)) break;
            const uint8_t* sR = smem + s * kStage + kBytesA;
            uint8_t* sB = smem + s * kStage + kBytesA + kBytesR;
            for (int job = ct; job < (kC / 8) * W; job += kConvWarps * 32) {
                const int h = job / W, c = job - h * W;
                const float4 a = *reinterpret_cast<const float4*>(sR + 2 * h * kSlot + c * 16);
                const float4 b = *reinterpret_cast<const float4*>(sR + (2 * h + 1) * kSlot + c * 16);
                const float f[8] = {a.x, a.y, a.z, a.w, b.x, b.y, b.z, b.w};
                uint32_t hi[4], lo[4];
#pragma unroll
                for (int e = 0; e < 4; ++e) {
                    hi[e] = pack_bf16(f[2 * e], f[2 * e + 1]);
                    lo[e] = pack_bf16(f[2 * e] - __uint_as_float(hi[e] << 16),
                                      f[2 * e + 1] - __uint_as_float(hi[e] & 0xFFFF0000u));
                }
                *reinterpret_cast<uint4*>(sB + h * kSlot + c * 16) = make_uint4(hi[0], hi[1], hi[2], hi[3]);
                *reinterpret_cast<uint4*>(sB + kBytesB + h * kSlot + c * 16) = make_uint4(lo[0], lo[1], lo[2], lo[3]);
            }
            asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
            __syncwarp();
            if (lane == 0) asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(gen_smem_u32(&full[s])) : "memory");
        }
    }
    __syncthreads();
    // all issued MMAs (they complete in order) before the accumulators are read or freed
    bool ok = true;
    if (tid == 0) {
        const int lm = last_mma;
        if (lm >= 0) {
            bool done = false;
            for (unsigned it = 0; it < tc::kWaitLimit && !done; ++it)
                done = gen_mbar_try_wait(gen_smem_u32(&empty[lm % kStages]), par(lm));
            if (!done) atomicExch(flag, 4);
            ok = done && lm == n - 1 && !abort_word;
        } else {
            ok = n == 0 && !abort_word;
        }
    }
    if (!__syncthreads_or(!ok)) {
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        // epilogue: job = (tile, lane quarter); a warp reads its own quarter (warp % 4)
        for (int job = warp; job < 24; job += kThreads / 32) {
            const int t = job >> 2, q = job & 3, dxi = t >> 1, pq = t & 1;
            if (pq == 1 && q < 2) continue;                 // tile Q's first half repeats tile P's
            const int row = q * 32 + lane, ci = row & 63, dy = pq + (row >> 6) - 1;
            float v[kC];
            if (n > 0) {
                const uint32_t taddr = tmem + ((uint32_t)(q * 32) << 16) + (uint32_t)(t * 64);
                tmem_ld16(taddr + 0, v);
                tmem_ld16(taddr + 16, v + 16);
                tmem_ld16(taddr + 32, v + 32);
                asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
            } else {
#pragma unroll
                for (int c = 0; c < kC; ++c) v[c] = 0.0f;
            }
            if (ci < kC) {
                const int r = ((dy + 1) * 3 + dxi) * kC + ci;
                float4* dst = reinterpret_cast<float4*>(part + ((size_t)blockIdx.x * 9 * kC + r) * kC);
#pragma unroll
                for (int c = 0; c < kC / 4; ++c) dst[c] = make_float4(v[4 * c], v[4 * c + 1], v[4 * c + 2], v[4 * c + 3]);
            }
        }
    } else if (tid == 0) {
        atomicExch(flag, 4);
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    if (warp == 0)
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(kCols) : "memory");
}

// Weight gradient: dW[tap][ci][co] = sum_p in[p + tap, ci] * dout[p, co], over the images and
// tiles given to one CTA; per-CTA partials go to `part` and are summed by k_gen_sum_parts.
// Thread layout: 9 taps x (CIN/6) ci groups x (COUT/8) co groups (6 x 8 accumulators each).
template <int CIN, int COUT>
__global__ void __launch_bounds__(432)
k_gen_wgrad(const __nv_bfloat16* __restrict__ in, const float* __restrict__ dout, float* __restrict__ part,
            int L, int images_per_cta, int nimg) {
    extern __shared__ float gsm[];
    constexpr int T2 = kTile + 2;
    constexpr int CG = (CIN + 5) / 6, OG = (COUT + 7) / 8;
    float* tin = gsm;                       // [T2*T2][CIN]
    float* tdo = gsm + T2 * T2 * CIN;       // [kTile*kTile][COUT]
    const int tiles_x = L / kTile;
    const int tile = blockIdx.x % (tiles_x * tiles_x);
    const int igrp = blockIdx.x / (tiles_x * tiles_x);
    const int ty0 = (tile / tiles_x) * kTile, tx0 = (tile % tiles_x) * kTile;
    const int t = threadIdx.x;
    const bool active = t < 9 * CG * OG;
    const int tap = t / (CG * OG), rr = t % (CG * OG), cg = rr / OG, og = rr % OG;
    const int dy = tap / 3, dx = tap % 3;
    float acc[6][8];
#pragma unroll
    for (int i = 0; i < 6; ++i)
#pragma unroll
        for (int j = 0; j < 8; ++j) acc[i][j] = 0.0f;
    for (int im = 0; im < images_per_cta; ++im) {
        const int img = igrp * images_per_cta + im;
        if (img >= nimg) break;
        const size_t ibase = (size_t)img * L * L;
        __syncthreads();
        // 16-byte loads (8 BF16 inputs, 4 FP32 gradients), several in flight per thread
        static_assert(CIN % 8 == 0 && COUT % 4 == 0, "16-byte staging");
        // chunk planes of this image; pixel index fastest, so consecutive threads read consecutive pixels
        const size_t LL = (size_t)L * L;
        const uint4* isrc = reinterpret_cast<const uint4*>(in + ibase * CIN);
        const float4* gsrc = reinterpret_cast<const float4*>(dout + ibase * COUT);
#pragma unroll 4
        for (int i = threadIdx.x; i < T2 * T2 * (CIN / 8); i += blockDim.x) {
            const int c8 = i / (T2 * T2), pix = i - c8 * T2 * T2, yy = pix / T2, xx = pix - yy * T2;
            int gy = ty0 + yy - 1, gx = tx0 + xx - 1;   // in [-1, L]: one wrap
            gy += (gy < 0) ? L : ((gy >= L) ? -L : 0);
            gx += (gx < 0) ? L : ((gx >= L) ? -L : 0);
            const uint4 q = __ldg(isrc + (size_t)c8 * LL + (size_t)gy * L + gx);
            const __nv_bfloat16* e = reinterpret_cast<const __nv_bfloat16*>(&q);
            float* d = tin + pix * CIN + c8 * 8;
#pragma unroll
            for (int k = 0; k < 8; ++k) d[k] = __bfloat162float(e[k]);
        }
#pragma unroll 4
        for (int i = threadIdx.x; i < kTile * kTile * (COUT / 4); i += blockDim.x) {
            const int c4 = i / (kTile * kTile), pix = i - c4 * kTile * kTile, yy = pix / kTile, xx = pix - yy * kTile;
            reinterpret_cast<float4*>(tdo + pix * COUT)[c4] =
                __ldg(gsrc + (size_t)c4 * LL + (size_t)(ty0 + yy) * L + tx0 + xx);
        }
        __syncthreads();
        if (active) {
            for (int py = 0; py < kTile; ++py)
                for (int px = 0; px < kTile; ++px) {
                    const float* xi = tin + ((py + dy) * T2 + px + dx) * CIN + cg * 6;
                    const float* go = tdo + (py * kTile + px) * COUT + og * 8;
                    float xv[6], gv[8];
#pragma unroll
                    for (int i = 0; i < 6; ++i) xv[i] = (cg * 6 + i < CIN) ? xi[i] : 0.0f;
#pragma unroll
                    for (int j = 0; j < 8; ++j) gv[j] = (og * 8 + j < COUT) ? go[j] : 0.0f;
#pragma unroll
                    for (int i = 0; i < 6; ++i)
#pragma unroll
                        for (int j = 0; j < 8; ++j) acc[i][j] = fmaf(xv[i], gv[j], acc[i][j]);
                }
        }
    }
    if (!active) return;
    float* dst = part + (size_t)blockIdx.x * 9 * CIN * COUT;
#pragma unroll
    for (int i = 0; i < 6; ++i)
#pragma unroll
        for (int j = 0; j < 8; ++j) {
            const int ci = cg * 6 + i, co = og * 8 + j;
            if (ci < CIN && co < COUT) dst[(tap * CIN + ci) * COUT + co] = acc[i][j];
        }
}

__global__ void k_gen_sum_parts(const float* __restrict__ part, int nparts, int n, float* __restrict__ out) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    float s = 0.0f;
    for (int p = 0; p < nparts; ++p) s += part[(size_t)p * n + i];
    out[i] = s;
}

// Sum of many partials for few outputs: block i adds part[0..nparts)[i], thread t the parts
// t, t + 128, ..., then a fixed-order tree (the same result on every run).
__global__ void __launch_bounds__(128)
k_gen_sum_parts_wide(const float* __restrict__ part, int nparts, int n, float* __restrict__ out) {
    __shared__ float red[128];
    const int i = blockIdx.x, t = threadIdx.x;
    float s = 0.0f;
    for (int p = t; p < nparts; p += 128) s += part[(size_t)p * n + i];
    red[t] = s;
    __syncthreads();
    for (int h = 64; h > 0; h >>= 1) {
        if (t < h) red[t] += red[t + h];
        __syncthreads();
    }
    if (t == 0) out[i] = red[0];
}

// Bias gradient, first stage: block b sums pixels [b*chunk, (b+1)*chunk) of the planar FP32
// dout (4 channels per 16-byte vector) into part[b][co]. Threads = channel group g x pixel
// lane; consecutive lanes read consecutive pixels of one group (coalesced 16-byte loads); the
// lanes are then added in a fixed order. The partials are summed by k_gen_sum_parts_wide.
__global__ void __launch_bounds__(256)
k_gen_bgrad_part(const float* __restrict__ dout, int npix, int LL, int cout, int chunk, float* __restrict__ part) {
    const int G = cout / 4, lanes = blockDim.x / G;
    const int t = threadIdx.x, g = t / lanes, pl = t - g * lanes;
    const int p0 = blockIdx.x * chunk, p1 = min(p0 + chunk, npix);
    float4 s = make_float4(0.f, 0.f, 0.f, 0.f);
    if (g < G) {
#pragma unroll 4
        for (int p = p0 + pl; p < p1; p += lanes) {
            const int img = p / LL, pp = p - img * LL;
            const float4 v = __ldg(reinterpret_cast<const float4*>(dout) + ((size_t)img * G + g) * LL + pp);
            s.x += v.x;
            s.y += v.y;
            s.z += v.z;
            s.w += v.w;
        }
    }
    __shared__ float4 red[256];
    red[t] = s;
    __syncthreads();
    if (t < cout) {
        const int gg = t / 4, e = t % 4;
        float v = 0.0f;
        for (int k = 0; k < lanes; ++k) {
            const float4 r = red[gg * lanes + k];
            v += e == 0 ? r.x : e == 1 ? r.y : e == 2 ? r.z : r.w;
        }
        part[(size_t)blockIdx.x * cout + t] = v;
    }
}

// BF16 copies of the weights: wb[tap][ci][co] and the flipped transpose wt[8-tap][co][ci].
__global__ void k_gen_cast(const float* __restrict__ w, int cin, int cout, __nv_bfloat16* __restrict__ wb,
                           __nv_bfloat16* __restrict__ wt) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= 9 * cin * cout) return;
    const int tap = i / (cin * cout), r = i - tap * cin * cout, ci = r / cout, co = r - ci * cout;
    const __nv_bfloat16 v = __float2bfloat16(w[i]);
    wb[i] = v;
    wt[((8 - tap) * cout + co) * cin + ci] = v;
}

__global__ void k_gen_adam(float* __restrict__ p, const float* __restrict__ g, float* __restrict__ m,
                           float* __restrict__ v, int n, float lr, float b1, float b2, float c1, float c2,
                           float eps) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float gi = g[i];
    const float mi = b1 * m[i] + (1.0f - b1) * gi;
    const float vi = b2 * v[i] + (1.0f - b2) * gi * gi;
    m[i] = mi;
    v[i] = vi;
    p[i] -= lr * (mi / c1) / (sqrtf(vi / c2) + eps);
}

// Network input for a batch: y = normalise(sqrt(1 - s^2) x + s g) and the condition channels.
// mode 0: x from the dataset (index per item), target = x.  mode 1: x = current estimate `cur`
// (sampling), g fresh noise from Philox (stream NOISE, counter = draws + item).  mode 2: as 1,
// but g is the noise predicted from the previous input y' at level s_prev,
// g = (y' - sqrt(1 - s_prev^2) x) / s_prev (deterministic DDIM-style update).  mode 3: the
// variance-preserving posterior step from y' at s_prev to level s (DDPM-style): with
// a' = 1 - s_prev^2, a = 1 - s^2, alpha = a'/a, y = sqrt(a)(1-alpha)/(1-a') x
// + sqrt(alpha)(1-a)/(1-a') y' + sqrt((1-a)(1-alpha)/(1-a')) g, then normalised.
__global__ void k_gen_input(int mode, const __nv_bfloat16* __restrict__ snaps, const int* __restrict__ idx,
                            const float* __restrict__ cur, const float* __restrict__ sig,
                            const float* __restrict__ cnd, int L, uint32_t k0, uint32_t k1,
                            unsigned long long draw0, __nv_bfloat16* __restrict__ act0,
                            float* __restrict__ target, float s_prev) {
    const int item = blockIdx.y;
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= L * L) return;
    float x[3];
    if (mode == 0) {
        const __nv_bfloat16* s = snaps + ((size_t)idx[item] * L * L + p) * 3;
        for (int c = 0; c < 3; ++c) x[c] = __bfloat162float(s[c]);
    } else {
        const float* s = cur + ((size_t)item * L * L + p) * kGenCout;
        for (int c = 0; c < 3; ++c) x[c] = s[c];
    }
    const float s = sig[item];
    const unsigned long long d = draw0 + (unsigned long long)item;
    nmmc_u4 r = nmmc_philox((uint32_t)p, (uint32_t)d, (uint32_t)(d >> 32) | (NMMC_STREAM_NOISE << 28), 0u, k0, k1);
    // Box-Muller: three normals from four uniforms
    const float u1 = nmmc_u01f(r.x), u2 = nmmc_u01f(r.y), u3 = nmmc_u01f(r.z), u4 = nmmc_u01f(r.w);
    const float rA = sqrtf(-2.0f * logf(u1)), rB = sqrtf(-2.0f * logf(u3));
    float sa, ca, sb, cb;
    sincospif(2.0f * u2, &sa, &ca);
    sincospif(2.0f * u4, &sb, &cb);
    float g[3] = {rA * ca, rA * sa, rB * cb};
    if (mode == 2 && s_prev < 1.0f) {
        const __nv_bfloat16* yp = act0 + ((size_t)item * L * L + p) * kGenCin0;
        const float kp = sqrtf(fmaxf(0.0f, 1.0f - s_prev * s_prev));
        for (int c = 0; c < 3; ++c) g[c] = (__bfloat162float(yp[c]) - kp * x[c]) / s_prev;
    }
    const float keep = sqrtf(fmaxf(0.0f, 1.0f - s * s));
    float y[3], n2 = 0.0f;
    if (mode == 3 && s_prev < 1.0f && s_prev > s) {
        const __nv_bfloat16* yp = act0 + ((size_t)item * L * L + p) * kGenCin0;
        const float ap = 1.0f - s_prev * s_prev, a = 1.0f - s * s, alpha = ap / a;
        const float cx = sqrtf(a) * (1.0f - alpha) / (1.0f - ap);
        const float cy = sqrtf(alpha) * (1.0f - a) / (1.0f - ap);
        const float cg = sqrtf(fmaxf(0.0f, (1.0f - a) * (1.0f - alpha) / (1.0f - ap)));
        for (int c = 0; c < 3; ++c) {
            y[c] = cx * x[c] + cy * __bfloat162float(yp[c]) + cg * g[c];
            n2 += y[c] * y[c];
        }
    } else {
        for (int c = 0; c < 3; ++c) {
            y[c] = keep * x[c] + s * g[c];
            n2 += y[c] * y[c];
        }
    }
    const float inv = n2 > 0.0f ? rsqrtf(n2) : 0.0f;
    __nv_bfloat16* a = act0 + ((size_t)item * L * L + p) * kGenCin0;
    for (int c = 0; c < 3; ++c) a[c] = __float2bfloat16(y[c] * inv);
    a[3] = __float2bfloat16(cnd[3 * item] / 1.5f);
    a[4] = __float2bfloat16(cnd[3 * item + 1]);
    a[5] = __float2bfloat16(cnd[3 * item + 2] / 0.8f);
    a[6] = __float2bfloat16(s);
    a[7] = __float2bfloat16(0.0f);
    if (mode == 0 && target) {
        float* t = target + ((size_t)item * L * L + p) * kGenCout;
        t[0] = x[0];
        t[1] = x[1];
        t[2] = x[2];
        t[3] = 0.0f;
    }
}

// Loss and its gradient through spin = v/|v|: loss += |s - x|^2 / npix_total;
// dL/dv = (g - s (s.g)) / |v| with g = 2 (s - x) / npix_total.
__global__ void k_gen_head(const float* __restrict__ v, const float* __restrict__ target, int npix, float scale,
                           float* __restrict__ gv, double* __restrict__ loss) {
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    float l = 0.0f;
    if (p < npix) {
        const float* a = v + (size_t)p * kGenCout;
        const float* x = target + (size_t)p * kGenCout;
        const float n2 = a[0] * a[0] + a[1] * a[1] + a[2] * a[2] + 1e-12f;
        const float inv = rsqrtf(n2);
        float s[3], g[3], sg = 0.0f;
        for (int c = 0; c < 3; ++c) {
            s[c] = a[c] * inv;
            const float d = s[c] - x[c];
            l += d * d;
            g[c] = 2.0f * d * scale;
            sg += s[c] * g[c];
        }
        float* o = gv + (size_t)p * kGenCout;
        for (int c = 0; c < 3; ++c) o[c] = (g[c] - s[c] * sg) * inv;
        o[3] = 0.0f;
    }
    for (int off = 16; off > 0; off >>= 1) l += __shfl_down_sync(0xffffffffu, l, off);
    if ((threadIdx.x & 31) == 0) atomicAdd(loss, (double)(l * scale));
}

// Sampling: cur <- normalise(v) (the denoised estimate)
__global__ void k_gen_normalise(const float* __restrict__ v, int npix, float* __restrict__ cur) {
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= npix) return;
    const float* a = v + (size_t)p * kGenCout;
    const float n2 = a[0] * a[0] + a[1] * a[1] + a[2] * a[2];
    const float inv = n2 > 0.0f ? rsqrtf(n2) : 0.0f;
    float* o = cur + (size_t)p * kGenCout;
    o[0] = a[0] * inv;
    o[1] = a[1] * inv;
    o[2] = a[2] * inv;
    o[3] = 0.0f;
}

// Sampler chain (split-colour FP32 planes, 2-D) <-> NHWC
__global__ void k_gen_from_chain(const DevModel m, const float* __restrict__ spins, const int* __restrict__ chains,
                                 __nv_bfloat16* __restrict__ snaps, int slot0) {
    const int item = blockIdx.y, chain = chains[item];
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    const int L = m.edge;
    if (p >= L * L) return;
    const int y = p / L, x = p - y * L, colour = (x + y) & 1;
    const size_t P = (size_t)m.nhalf_pad, i = (size_t)y * m.hx + (x >> 1);
    const float* pl = spins + ((size_t)chain * 2 + colour) * 3 * P;
    __nv_bfloat16* o = snaps + ((size_t)(slot0 + item) * L * L + p) * 3;
    o[0] = __float2bfloat16(pl[i]);
    o[1] = __float2bfloat16(pl[P + i]);
    o[2] = __float2bfloat16(pl[2 * P + i]);
}

__global__ void k_gen_to_chain(const DevModel m, float* __restrict__ spins, const int* __restrict__ chains,
                               const float* __restrict__ cur) {
    const int item = blockIdx.y, chain = chains[item];
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    const int L = m.edge;
    if (p >= L * L) return;
    const int y = p / L, x = p - y * L, colour = (x + y) & 1;
    const size_t P = (size_t)m.nhalf_pad, i = (size_t)y * m.hx + (x >> 1);
    float* pl = spins + ((size_t)chain * 2 + colour) * 3 * P;
    const float* a = cur + ((size_t)item * L * L + p) * kGenCout;
    pl[i] = a[0];
    pl[P + i] = a[1];
    pl[2 * P + i] = a[2];
}

// ------------------------------------------------------------------------------------------
// host side
// ------------------------------------------------------------------------------------------
namespace {

// Raises a kernel's dynamic shared-memory limit on the generator's device (once per size);
// max_shared also asks for the whole L1/shared array as shared memory.
int ensure_smem(nmmc_gen* g, const void* fn, int bytes, bool max_shared) {
    auto it = g->attr_smem.find(fn);
    if (it != g->attr_smem.end() && it->second >= bytes) return NMMC_OK;
    cudaError_t e = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
    if (e == cudaSuccess && max_shared)
        e = cudaFuncSetAttribute(fn, cudaFuncAttributePreferredSharedMemoryCarveout, (int)cudaSharedmemCarveoutMaxShared);
    if (e != cudaSuccess) return cuda_check(e, "cudaFuncSetAttribute(generator kernel)");
    g->attr_smem[fn] = bytes;
    return NMMC_OK;
}

template <int CIN, int COUT, typename TIN, int EPI>
int conv_launch(nmmc_gen* g, const TIN* in, const __nv_bfloat16* w, const float* bias,
                const __nv_bfloat16* mask, int mask_c, void* out, int nimg) {
    const size_t smem = (size_t)(9 * CIN * COUT + CIN * (kTile + 2) * (kTile + 2)) * sizeof(float);
    if (int rc = ensure_smem(g, (const void*)k_gen_conv<CIN, COUT, TIN, EPI>, (int)smem, false)) return rc;
    dim3 grid(g->L / kTile, g->L / kTile, nimg);
    k_gen_conv<CIN, COUT, TIN, EPI><<<grid, 256, smem, g->stream>>>(in, w, bias, mask, mask_c, out, g->L);
    return cuda_check(cudaGetLastError(), "k_gen_conv");
}

// Hidden-layer convolution on the tensor cores: persistent CTAs, as many per SM as the shared
// memory allows (two for the BF16 modes at L = 128, one for the TF32 data gradient).
// cuTensorMapEncodeTiled through the runtime's driver entry point (no link against libcuda).
using EncodeTiledFn = CUresult (*)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                                   const cuuint64_t*, const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave,
                                   CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);
static EncodeTiledFn encode_tiled() {
    static const EncodeTiledFn fn = []() -> EncodeTiledFn {
        void* p = nullptr;
        cudaDriverEntryPointQueryResult q = cudaDriverEntryPointSymbolNotFound;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) != cudaSuccess ||
            q != cudaDriverEntryPointSuccess)
            return nullptr;
        return (EncodeTiledFn)p;
    }();
    return fn;
}

// Tensor map of chunk-planar activations [nimg][ICH][L][L][epc] (ICH chunks of epc channels)
// for the TMA-fed convolutions (L = 128): dimensions (element of a chunk, x, y, chunk, image),
// so that one box [epc, 130, 1, 1, 1] at x = -1 is one (row, chunk) block of a window, 2080
// contiguous bytes of which the two edge positions fall outside the row and are zero-filled.
template <int MODE, int ICH = tc::chunks<MODE>()>
int window_map(const typename tc::Traits<MODE>::TA* in, int L, int nimg, CUtensorMap* map) {
    const EncodeTiledFn enc = encode_tiled();
    if (!enc) return set_error(NMMC_ERR_CUDA, "cuTensorMapEncodeTiled is not available");
    constexpr int kEpc = tc::Traits<MODE>::kEpc, kCh = ICH;
    const cuuint64_t l = (cuuint64_t)L;
    const cuuint64_t dims[5] = {(cuuint64_t)kEpc, l, l, (cuuint64_t)kCh, (cuuint64_t)nimg};
    const cuuint64_t strides[4] = {16, 16ull * l, 16ull * l * l, 16ull * kCh * l * l};
    const cuuint32_t box[5] = {(cuuint32_t)kEpc, (cuuint32_t)tma::kSlots, 1, 1, 1};
    const cuuint32_t estr[5] = {1, 1, 1, 1, 1};
    const CUresult r = enc(map, MODE == 2 ? CU_TENSOR_MAP_DATA_TYPE_FLOAT32 : CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 5,
                           (void*)in, dims, strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE,
                           CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
                           CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) return set_error(NMMC_ERR_CUDA, "cuTensorMapEncodeTiled failed (%d)", (int)r);
    return NMMC_OK;
}

// single-role TMA kernel (every mode and layer shape; the data gradient's TF32 window leaves
// room for one stage). Forward layers take tiles of NMMC_GEN_OPT_TILE_ROWS output rows (default
// 2), the TF32 data gradient one.
template <int MODE, int ICH, int KCH, int CO, int R>
int conv_tma_launch_r(nmmc_gen* g, const CUtensorMap& map, const __nv_bfloat16* w, const uint8_t* wimg,
                      const float* bias, const __nv_bfloat16* mask, void* out, int nimg) {
    const int smem = tma::smem_bytes<MODE, ICH, KCH, CO, R>();
    if (int rc = ensure_smem(g, (const void*)k_gen_conv_tma<MODE, ICH, KCH, CO, R>, smem, true)) return rc;
    const int per_sm = std::max(1, std::min(2, g->smem_per_sm / (smem + 2048)));
    const int ntiles = nimg * g->L / R;
    const int grid = std::min(ntiles, per_sm * g->sm_count);
    k_gen_conv_tma<MODE, ICH, KCH, CO, R><<<grid, 128, smem, g->stream>>>(map, w, wimg, bias, mask, out, ntiles,
                                                                          g->d_flag);
    return cuda_check(cudaGetLastError(), "k_gen_conv_tma");
}

// wimg: the layer's weight image (forward modes; nullptr: the threads rearrange w)
template <int MODE, int ICH = tc::chunks<MODE>(), int KCH = ICH, int CO = tc::kC>
int conv_tma_launch(nmmc_gen* g, const typename tc::Traits<MODE>::TA* in, const __nv_bfloat16* w, const float* bias,
                    const __nv_bfloat16* mask, void* out, int nimg, const uint8_t* wimg = nullptr) {
    alignas(64) CUtensorMap map;
    if (int rc = window_map<MODE, ICH>(in, g->L, nimg, &map)) return rc;
    if (MODE == 2 || !g->use_wimg) wimg = nullptr;
    if constexpr (MODE != 2)
        if (g->tile_rows == 2) return conv_tma_launch_r<MODE, ICH, KCH, CO, 2>(g, map, w, wimg, bias, mask, out, nimg);
    return conv_tma_launch_r<MODE, ICH, KCH, CO, 1>(g, map, w, wimg, bias, mask, out, nimg);
}

// The first (8 -> 48, ReLU) and last (48 -> 4, linear) layers on the tensor cores when L = 128
// and the TMA path is on; false when they run on the FMA pipes.
bool edge_layers_on_tc(const nmmc_gen* g) { return g->use_tc && g->use_tma && g->L == tc::kM; }

// warp-specialised TMA kernel (BF16 modes), one CTA per SM
template <int MODE>
int conv_tmaws_launch(nmmc_gen* g, const __nv_bfloat16* in, const __nv_bfloat16* w, const float* bias, void* out,
                      int nimg) {
    alignas(64) CUtensorMap map;
    if (int rc = window_map<MODE>(in, g->L, nimg, &map)) return rc;
    const int smem = tmaws_smem_bytes<MODE>();
    if (int rc = ensure_smem(g, (const void*)k_gen_conv_tmaws<MODE>, smem, true)) return rc;
    const int ntiles = nimg * g->L;
    const int grid = std::min(ntiles, g->sm_count);
    k_gen_conv_tmaws<MODE><<<grid, kTwsThreads, smem, g->stream>>>(map, w, bias, out, ntiles, g->d_flag);
    return cuda_check(cudaGetLastError(), "k_gen_conv_tmaws");
}

template <int MODE>
int conv_tc_launch(nmmc_gen* g, const typename tc::Traits<MODE>::TA* in, const __nv_bfloat16* w, const float* bias,
                   const __nv_bfloat16* mask, void* out, int nimg, const uint8_t* wimg = nullptr) {
    if (g->use_tma && g->L == tc::kM && !(MODE != 2 && g->use_ws)) {
        if constexpr (MODE != 2)
            if (g->use_tma == 2) return conv_tmaws_launch<MODE>(g, in, w, bias, out, nimg);
        return conv_tma_launch<MODE>(g, in, w, bias, mask, out, nimg, wimg);
    }
    if constexpr (MODE != 2) {   // BF16 modes: the warp-specialised kernel when two windows fit
        const int ws = ws_smem_bytes<MODE>(g->L);
        if (g->use_ws && ws <= tc::kSmemMax) {
            if (int rc = ensure_smem(g, (const void*)k_gen_conv_ws<MODE>, ws, true)) return rc;
            const int tiles_per_img = (g->L * (g->L + 2) + tc::kM - 1) / tc::kM;
            const int ntiles = nimg * tiles_per_img;
            const int grid = std::min(ntiles, g->sm_count);
            k_gen_conv_ws<MODE><<<grid, kWsThreads, ws, g->stream>>>(in, w, bias, out, g->L, tiles_per_img, ntiles,
                                                                      g->d_flag);
            return cuda_check(cudaGetLastError(), "k_gen_conv_ws");
        }
    }
    const int smem = tc::smem_bytes<MODE>(g->L);
    if (smem > tc::kSmemMax)
        return set_error(NMMC_ERR_UNSUPPORTED, "lattice edge %d too large for the tensor-core convolution", g->L);
    // the whole unified L1/shared array as shared memory, so two BF16 CTAs fit per SM
    if (int rc = ensure_smem(g, (const void*)k_gen_conv_tc<MODE>, smem, true)) return rc;
    // CTAs per SM from the shared memory (+ static and the 1 KB the driver reserves), at most two
    // (64 TMEM columns and 128 threads each). The runtime's occupancy query answers 1 for this
    // kernel on GB300 although two CTAs are co-resident when launched.
    const int per_sm = std::max(1, std::min(2, g->smem_per_sm / (smem + 2048)));
    const int tiles_per_img = (g->L * (g->L + 2) + tc::kM - 1) / tc::kM;   // padded rows 1..L
    const int ntiles = nimg * tiles_per_img;
    const int grid = std::min(ntiles, per_sm * g->sm_count);
    k_gen_conv_tc<MODE><<<grid, 128, smem, g->stream>>>(in, w, bias, mask, out, g->L, tiles_per_img, ntiles, g->d_flag);
    return cuda_check(cudaGetLastError(), "k_gen_conv_tc");
}

// Reads and clears the device error word after the stream has drained.
int check_flag(nmmc_gen* g) {
    int f = 0;
    NMMC_CUDA(cudaMemcpy(&f, g->d_flag, sizeof(int), cudaMemcpyDeviceToHost));
    if (!f) return NMMC_OK;
    cudaMemset(g->d_flag, 0, sizeof(int));
    return set_error(NMMC_ERR_TIMEOUT, "a tensor-core convolution gave up waiting for its MMAs (code %d)", f);
}

// Hidden-layer weight gradient on the tensor cores (k_gen_wgrad_tc): as many CTAs as SMs (one
// per SM), as the partial scratch holds and as there are K-blocks.
int wgrad_tc_launch(nmmc_gen* g, const __nv_bfloat16* in, const float* dout, float* gw, int nimg) {
    const size_t n = (size_t)9 * tc::kC * tc::kC;
    const int W = wg::block_len(g->L);
    const int nkb = (int)((size_t)nimg * g->L * (g->L / W));
    const int nparts = (int)std::min<size_t>({(size_t)nkb, (size_t)std::max(1, g->sm_count), g->wpart_cap / n});
    if (nparts < 1) return set_error(NMMC_ERR_ARG, "weight-gradient scratch too small");
    const void* fn = W == 64 ? (const void*)k_gen_wgrad_tc<4>
                   : W == 48 ? (const void*)k_gen_wgrad_tc<3>
                   : W == 32 ? (const void*)k_gen_wgrad_tc<2> : (const void*)k_gen_wgrad_tc<1>;
    if (int rc = ensure_smem(g, fn, (int)wg::kSmem, true)) return rc;
    if (W == 64)
        k_gen_wgrad_tc<4><<<nparts, wg::kThreads, wg::kSmem, g->stream>>>(in, dout, g->wpart, g->L, nkb, g->d_flag);
    else if (W == 48)
        k_gen_wgrad_tc<3><<<nparts, wg::kThreads, wg::kSmem, g->stream>>>(in, dout, g->wpart, g->L, nkb, g->d_flag);
    else if (W == 32)
        k_gen_wgrad_tc<2><<<nparts, wg::kThreads, wg::kSmem, g->stream>>>(in, dout, g->wpart, g->L, nkb, g->d_flag);
    else
        k_gen_wgrad_tc<1><<<nparts, wg::kThreads, wg::kSmem, g->stream>>>(in, dout, g->wpart, g->L, nkb, g->d_flag);
    k_gen_sum_parts<<<(int)((n + 255) / 256), 256, 0, g->stream>>>(g->wpart, nparts, (int)n, gw);
    return cuda_check(cudaGetLastError(), "k_gen_wgrad_tc");
}

template <int CIN, int COUT>
int wgrad_launch(nmmc_gen* g, const __nv_bfloat16* in, const float* dout, float* gw, int nimg) {
    if (CIN == tc::kC && COUT == tc::kC && g->use_tc && wg::block_len(g->L) > 0)
        return wgrad_tc_launch(g, in, dout, gw, nimg);
    const int tiles = (g->L / kTile) * (g->L / kTile);
    const int per = 4;
    const int groups = (nimg + per - 1) / per;
    const int nparts = tiles * groups;
    const size_t n = (size_t)9 * CIN * COUT;
    if ((size_t)nparts * n > g->wpart_cap) return set_error(NMMC_ERR_ARG, "weight-gradient scratch too small");
    const size_t smem = (size_t)((kTile + 2) * (kTile + 2) * CIN + kTile * kTile * COUT) * sizeof(float);
    if (int rc = ensure_smem(g, (const void*)k_gen_wgrad<CIN, COUT>, (int)smem, false)) return rc;
    k_gen_wgrad<CIN, COUT><<<nparts, 432, smem, g->stream>>>(in, dout, g->wpart, g->L, per, nimg);
    k_gen_sum_parts<<<(int)((n + 255) / 256), 256, 0, g->stream>>>(g->wpart, nparts, (int)n, gw);
    return cuda_check(cudaGetLastError(), "k_gen_wgrad");
}

// Bias gradient gb[co] = sum over the batch's pixels of dout[p, co] (wpart as scratch).
int bgrad_launch(nmmc_gen* g, const float* dout, int npix, int cout, float* gb) {
    // about two blocks per SM, chunks a multiple of 64 pixels
    const int per = (npix + 2 * std::max(1, g->sm_count) - 1) / (2 * std::max(1, g->sm_count));
    const int chunk = std::max(64, (per + 63) / 64 * 64);
    const int nblk = (npix + chunk - 1) / chunk;
    if (cout % 4 != 0 || cout > 256) return set_error(NMMC_ERR_ARG, "bias gradient: channels not a multiple of 4");
    if ((size_t)nblk * cout > g->wpart_cap) return set_error(NMMC_ERR_ARG, "bias-gradient scratch too small");
    k_gen_bgrad_part<<<nblk, 256, 0, g->stream>>>(dout, npix, g->L * g->L, cout, chunk, g->wpart);
    k_gen_sum_parts_wide<<<cout, 128, 0, g->stream>>>(g->wpart, nblk, cout, gb);
    return cuda_check(cudaGetLastError(), "k_gen_bgrad_part");
}

// One layer's BF16 weights wb[tap][k][n] in the B-operand layout k_gen_conv_tma uses in shared
// memory: per tap, NN/8 x KCH core matrices of 8 rows (n) x 16 bytes (8 consecutive k), zeros past
// cin and cout (KCH chunks of 8 inputs, NN outputs rounded up to 16).
template <int KCH, int NN>
__global__ void k_gen_wimage(const __nv_bfloat16* __restrict__ wb, int cin, int cout, uint8_t* __restrict__ img) {
    constexpr int KK = KCH * 8, kBT = (NN / 8) * KCH * tc::kCore;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= 9 * NN * KK) return;
    const int tap = i / (NN * KK), r = i - tap * NN * KK, nn = r / KK, k = r - nn * KK;
    const __nv_bfloat16 v = (nn < cout && k < cin) ? wb[(tap * cin + k) * cout + nn] : __float2bfloat16(0.0f);
    *reinterpret_cast<__nv_bfloat16*>(img + tap * kBT + ((nn >> 3) * KCH + k / 8) * tc::kCore + (nn & 7) * 16 +
                                      (k % 8) * 2) = v;
}

int refresh_weights(nmmc_gen* g) {
    for (int l = 0; l < kGenLayers; ++l) {
        GenLayer& y = g->layer[l];
        const int n = (int)y.nw();
        k_gen_cast<<<(n + 255) / 256, 256, 0, g->stream>>>(y.w, y.cin, y.cout, y.wb, y.wt);
        // the images of the TMA kernel's layer shapes: first 8 -> 48 (K of two chunks), hidden
        // 48 -> 48, last 48 -> 4 (N = 16)
        if (l == 0)
            k_gen_wimage<2, tma::nmma(kGenC)><<<(9 * 48 * 16 + 255) / 256, 256, 0, g->stream>>>(y.wb, y.cin, y.cout, y.wimg);
        else if (l == kGenLayers - 1)
            k_gen_wimage<6, tma::nmma(kGenCout)><<<(9 * 16 * 48 + 255) / 256, 256, 0, g->stream>>>(y.wb, y.cin, y.cout,
                                                                                                  y.wimg);
        else
            k_gen_wimage<6, tma::nmma(kGenC)><<<(9 * 48 * 48 + 255) / 256, 256, 0, g->stream>>>(y.wb, y.cin, y.cout, y.wimg);
    }
    return cuda_check(cudaGetLastError(), "k_gen_cast");
}

int ensure_batch(nmmc_gen* g, int b) {
    if (b <= g->bcap) return NMMC_OK;
    for (int l = 0; l < kGenLayers; ++l) cudaFree(g->act[l]);
    cudaFree(g->vout);
    cudaFree(g->target);
    cudaFree(g->g0);
    cudaFree(g->g1);
    cudaFree(g->gv);
    cudaFree(g->wpart);
    cudaFree(g->d_idx);
    cudaFree(g->d_sig);
    cudaFree(g->d_cnd);
    const size_t np = (size_t)b * g->L * g->L;
    NMMC_CUDA(cudaMalloc(&g->act[0], np * kGenCin0 * sizeof(__nv_bfloat16)));
    for (int l = 1; l < kGenLayers; ++l) NMMC_CUDA(cudaMalloc(&g->act[l], np * kGenC * sizeof(__nv_bfloat16)));
    NMMC_CUDA(cudaMalloc(&g->vout, np * kGenCout * sizeof(float)));
    NMMC_CUDA(cudaMalloc(&g->target, np * kGenCout * sizeof(float)));
    NMMC_CUDA(cudaMalloc(&g->g0, np * kGenC * sizeof(float)));
    NMMC_CUDA(cudaMalloc(&g->g1, np * kGenC * sizeof(float)));
    NMMC_CUDA(cudaMalloc(&g->gv, np * kGenCout * sizeof(float)));
    const int tiles = (g->L / kTile) * (g->L / kTile);
    g->wpart_cap = (size_t)tiles * ((b + 3) / 4) * 9 * kGenC * kGenC;
    NMMC_CUDA(cudaMalloc(&g->wpart, g->wpart_cap * sizeof(float)));
    NMMC_CUDA(cudaMalloc(&g->d_idx, sizeof(int) * b));
    NMMC_CUDA(cudaMalloc(&g->d_sig, sizeof(float) * b));
    NMMC_CUDA(cudaMalloc(&g->d_cnd, sizeof(float) * 3 * b));
    g->bcap = b;
    return NMMC_OK;
}

// forward pass of nb images from act[0]; leaves act[1..7] and vout
int forward(nmmc_gen* g, int nb) {
    int rc;
    GenLayer* y = g->layer;
    rc = edge_layers_on_tc(g)
             ? conv_tma_launch<0, 1, 2, kGenC>(g, g->act[0], y[0].wb, y[0].b, nullptr, g->act[1], nb, y[0].wimg)
             : conv_launch<kGenCin0, kGenC, __nv_bfloat16, 0>(g, g->act[0], y[0].wb, y[0].b, nullptr, 0, g->act[1], nb);
    if (rc) return rc;
    for (int l = 1; l < kGenLayers - 1; ++l) {
        rc = g->use_tc ? conv_tc_launch<0>(g, g->act[l], y[l].wb, y[l].b, nullptr, g->act[l + 1], nb, y[l].wimg)
                       : conv_launch<kGenC, kGenC, __nv_bfloat16, 0>(g, g->act[l], y[l].wb, y[l].b, nullptr, 0,
                                                                    g->act[l + 1], nb);
        if (rc) return rc;
    }
    const GenLayer& yl = y[kGenLayers - 1];
    if (edge_layers_on_tc(g))
        return conv_tma_launch<3, 6, 6, kGenCout>(g, g->act[kGenLayers - 1], yl.wb, yl.b, nullptr, g->vout, nb,
                                                  yl.wimg);
    return conv_launch<kGenC, kGenCout, __nv_bfloat16, 1>(g, g->act[kGenLayers - 1], yl.wb, yl.b, nullptr, 0, g->vout, nb);
}

// backward from gv (dL/dv): fills gw/gb of every layer
int backward(nmmc_gen* g, int nb) {
    int rc;
    GenLayer* y = g->layer;
    const int npix = nb * g->L * g->L;
    const int last = kGenLayers - 1;
    // last layer: weights and bias, then data gradient into g0 (masked by act[last] > 0)
    if ((rc = wgrad_launch<kGenC, kGenCout>(g, g->act[last], g->gv, y[last].gw, nb))) return rc;
    if ((rc = bgrad_launch(g, g->gv, npix, kGenCout, y[last].gb))) return rc;
    if ((rc = conv_launch<kGenCout, kGenC, float, 2>(g, g->gv, y[last].wt, nullptr, g->act[last], kGenC, g->g0, nb)))
        return rc;
    float* cur = g->g0;
    float* nxt = g->g1;
    for (int l = last - 1; l >= 1; --l) {
        if ((rc = wgrad_launch<kGenC, kGenC>(g, g->act[l], cur, y[l].gw, nb))) return rc;
        if ((rc = bgrad_launch(g, cur, npix, kGenC, y[l].gb))) return rc;
        rc = g->use_tc ? conv_tc_launch<2>(g, cur, y[l].wt, nullptr, g->act[l], nxt, nb)
                       : conv_launch<kGenC, kGenC, float, 2>(g, cur, y[l].wt, nullptr, g->act[l], kGenC, nxt, nb);
        if (rc) return rc;
        float* t = cur;
        cur = nxt;
        nxt = t;
    }
    if ((rc = wgrad_launch<kGenCin0, kGenC>(g, g->act[0], cur, y[0].gw, nb))) return rc;
    if ((rc = bgrad_launch(g, cur, npix, kGenC, y[0].gb))) return rc;
    return cuda_check(cudaGetLastError(), "backward");
}

void free_gen(nmmc_gen* g) {
    if (!g) return;
    for (int l = 0; l < kGenLayers; ++l) {
        GenLayer& y = g->layer[l];
        cudaFree(y.w);
        cudaFree(y.b);
        cudaFree(y.wb);
        cudaFree(y.wt);
        cudaFree(y.wimg);
        cudaFree(y.gw);
        cudaFree(y.gb);
        cudaFree(y.mw);
        cudaFree(y.vw);
        cudaFree(y.mb);
        cudaFree(y.vb);
        cudaFree(g->act[l]);
    }
    cudaFree(g->snaps);
    cudaFree(g->cond);
    cudaFree(g->vout);
    cudaFree(g->target);
    cudaFree(g->g0);
    cudaFree(g->g1);
    cudaFree(g->gv);
    cudaFree(g->wpart);
    cudaFree(g->d_idx);
    cudaFree(g->d_sig);
    cudaFree(g->d_cnd);
    cudaFree(g->d_loss);
    cudaFree(g->d_flag);
    if (g->stream) cudaStreamDestroy(g->stream);
    delete g;
}

}  // namespace
}  // namespace nmmc

using namespace nmmc;
struct nmmc_ctx : public nmmc::Ctx {};

extern "C" {

int nmmc_gen_create(int L, int capacity, uint64_t seed, nmmc_gen** out) {
    if (!out || L < kTile || L % kTile || capacity < 0) return set_error(NMMC_ERR_ARG, "L must be a multiple of 16");
    *out = nullptr;
    nmmc_gen* g = new nmmc_gen();
    g->L = L;
    g->seed = seed;
    g->cap = capacity;
#define NMMC_GTRY(call)                                  \
    do {                                                 \
        cudaError_t _e = (call);                         \
        if (_e != cudaSuccess) {                         \
            int _rc = cuda_check(_e, #call);             \
            free_gen(g);                                 \
            return _rc;                                  \
        }                                                \
    } while (0)
    NMMC_GTRY(cudaStreamCreateWithFlags(&g->stream, cudaStreamNonBlocking));
    // He-style initialisation from Philox (host)
    for (int l = 0; l < kGenLayers; ++l) {
        GenLayer& y = g->layer[l];
        y.cin = (l == 0) ? kGenCin0 : kGenC;
        y.cout = (l == kGenLayers - 1) ? kGenCout : kGenC;
        const size_t n = y.nw();
        std::vector<float> w(n), b(y.cout, 0.0f);
        const float sd = sqrtf(2.0f / (9.0f * y.cin)) * (l == kGenLayers - 1 ? 0.5f : 1.0f);
        for (size_t i = 0; i < n; ++i) {
            nmmc_u4 r = nmmc_philox((uint32_t)i, (uint32_t)l, NMMC_STREAM_NOISE << 28, 7u, (uint32_t)seed,
                                    (uint32_t)(seed >> 32));
            const double u1 = ((double)r.x + 0.5) / 4294967296.0, u2 = ((double)r.y + 0.5) / 4294967296.0;
            w[i] = (float)(sd * sqrt(-2.0 * log(u1)) * cos(2.0 * M_PI * u2));
            const int co = (int)(i % y.cout);
            if (l == kGenLayers - 1 && co == 3) w[i] = 0.0f;   // padding channel
        }
        NMMC_GTRY(cudaMalloc(&y.w, n * sizeof(float)));
        NMMC_GTRY(cudaMalloc(&y.b, y.cout * sizeof(float)));
        NMMC_GTRY(cudaMalloc(&y.wb, n * sizeof(__nv_bfloat16)));
        NMMC_GTRY(cudaMalloc(&y.wt, n * sizeof(__nv_bfloat16)));
        NMMC_GTRY(cudaMalloc(&y.wimg, kWimgBytes));
        NMMC_GTRY(cudaMalloc(&y.gw, n * sizeof(float)));
        NMMC_GTRY(cudaMalloc(&y.gb, y.cout * sizeof(float)));
        NMMC_GTRY(cudaMalloc(&y.mw, n * sizeof(float)));
        NMMC_GTRY(cudaMalloc(&y.vw, n * sizeof(float)));
        NMMC_GTRY(cudaMalloc(&y.mb, y.cout * sizeof(float)));
        NMMC_GTRY(cudaMalloc(&y.vb, y.cout * sizeof(float)));
        NMMC_GTRY(cudaMemcpy(y.w, w.data(), n * sizeof(float), cudaMemcpyHostToDevice));
        NMMC_GTRY(cudaMemcpy(y.b, b.data(), y.cout * sizeof(float), cudaMemcpyHostToDevice));
        NMMC_GTRY(cudaMemset(y.mw, 0, n * sizeof(float)));
        NMMC_GTRY(cudaMemset(y.vw, 0, n * sizeof(float)));
        NMMC_GTRY(cudaMemset(y.mb, 0, y.cout * sizeof(float)));
        NMMC_GTRY(cudaMemset(y.vb, 0, y.cout * sizeof(float)));
    }
    if (capacity > 0) {
        NMMC_GTRY(cudaMalloc(&g->snaps, (size_t)capacity * L * L * 3 * sizeof(__nv_bfloat16)));
        NMMC_GTRY(cudaMalloc(&g->cond, (size_t)capacity * 3 * sizeof(float)));
    }
    NMMC_GTRY(cudaMalloc(&g->d_loss, sizeof(double)));
    NMMC_GTRY(cudaMalloc(&g->d_flag, sizeof(int)));
    NMMC_GTRY(cudaMemset(g->d_flag, 0, sizeof(int)));
    {
        int dev = 0;
        NMMC_GTRY(cudaGetDevice(&dev));
        NMMC_GTRY(cudaDeviceGetAttribute(&g->sm_count, cudaDevAttrMultiProcessorCount, dev));
        NMMC_GTRY(cudaDeviceGetAttribute(&g->smem_per_sm, cudaDevAttrMaxSharedMemoryPerMultiprocessor, dev));
    }
#undef NMMC_GTRY
    int rc = refresh_weights(g);
    if (!rc) rc = cuda_check(cudaStreamSynchronize(g->stream), "nmmc_gen_create");
    if (rc) {
        free_gen(g);
        return rc;
    }
    *out = g;
    return NMMC_OK;
}

void nmmc_gen_destroy(nmmc_gen* g) {
    if (g) cudaStreamSynchronize(g->stream);
    free_gen(g);
}

int nmmc_gen_param_count(const nmmc_gen* g) {
    if (!g) return 0;
    size_t n = 0;
    for (int l = 0; l < kGenLayers; ++l) n += g->layer[l].nw() + g->layer[l].cout;
    return (int)n;
}

// parameters in layer order: W [9][cin][cout] then b [cout]
int nmmc_gen_get_params(nmmc_gen* g, float* out, int n) {
    if (!g || !out || n != nmmc_gen_param_count(g)) return set_error(NMMC_ERR_ARG, "bad parameter buffer");
    NMMC_CUDA(cudaStreamSynchronize(g->stream));
    size_t o = 0;
    for (int l = 0; l < kGenLayers; ++l) {
        GenLayer& y = g->layer[l];
        NMMC_CUDA(cudaMemcpy(out + o, y.w, y.nw() * sizeof(float), cudaMemcpyDeviceToHost));
        o += y.nw();
        NMMC_CUDA(cudaMemcpy(out + o, y.b, y.cout * sizeof(float), cudaMemcpyDeviceToHost));
        o += y.cout;
    }
    return NMMC_OK;
}

int nmmc_gen_set_params(nmmc_gen* g, const float* in, int n) {
    if (!g || !in || n != nmmc_gen_param_count(g)) return set_error(NMMC_ERR_ARG, "bad parameter buffer");
    NMMC_CUDA(cudaStreamSynchronize(g->stream));
    size_t o = 0;
    for (int l = 0; l < kGenLayers; ++l) {
        GenLayer& y = g->layer[l];
        NMMC_CUDA(cudaMemcpy(y.w, in + o, y.nw() * sizeof(float), cudaMemcpyHostToDevice));
        o += y.nw();
        NMMC_CUDA(cudaMemcpy(y.b, in + o, y.cout * sizeof(float), cudaMemcpyHostToDevice));
        o += y.cout;
    }
    return refresh_weights(g);
}

// Snapshots of 2-D Heisenberg chains of `ctx` (edge == generator L) with their (T, B, D).
int nmmc_gen_add_snapshots(nmmc_gen* g, nmmc_ctx* c, const int* chains, int n, const double* cond) {
    if (!g || !c || !chains || !cond || n <= 0) return set_error(NMMC_ERR_ARG, "bad argument");
    if (c->dim != 2 || c->ising || c->edge != g->L || c->masked)
        return set_error(NMMC_ERR_UNSUPPORTED, "snapshots must come from unmasked 2-D Heisenberg lattices of edge %d", g->L);
    if (g->count + n > g->cap) return set_error(NMMC_ERR_ARG, "dataset capacity %d exceeded", g->cap);
    for (int i = 0; i < n; ++i)
        if (chains[i] < 0 || chains[i] >= c->nchains) return set_error(NMMC_ERR_ARG, "chain index out of range");
    DeviceScratch ds;
    int* d_ch = nullptr;
    NMMC_CUDA(ds.alloc(&d_ch, sizeof(int) * n));
    std::vector<float> cf(3 * (size_t)n);
    for (size_t i = 0; i < cf.size(); ++i) cf[i] = (float)cond[i];
    NMMC_CUDA(cudaStreamSynchronize(c->stream));
    NMMC_CUDA(cudaMemcpy(d_ch, chains, sizeof(int) * n, cudaMemcpyHostToDevice));
    NMMC_CUDA(cudaMemcpy(g->cond + 3 * (size_t)g->count, cf.data(), cf.size() * sizeof(float), cudaMemcpyHostToDevice));
    dim3 grid((g->L * g->L + 255) / 256, n);
    k_gen_from_chain<<<grid, 256, 0, g->stream>>>(c->m, (const float*)c->d_spins, d_ch, g->snaps, g->count);
    int rc = cuda_check(cudaStreamSynchronize(g->stream), "k_gen_from_chain");
    if (rc) return rc;
    g->count += n;
    return NMMC_OK;
}

int nmmc_gen_dataset_size(const nmmc_gen* g) { return g ? g->count : 0; }

// One optimisation step per batch: idx[b] snapshot indices, sig[b] noise levels. Returns the
// batch loss. lr <= 0 computes loss and gradients without updating (gradient checks).
int nmmc_gen_train_step(nmmc_gen* g, const int* idx, const float* sig, int nb, float lr, double* loss) {
    if (!g || !idx || !sig || nb <= 0) return set_error(NMMC_ERR_ARG, "bad argument");
    for (int i = 0; i < nb; ++i)
        if (idx[i] < 0 || idx[i] >= g->count) return set_error(NMMC_ERR_ARG, "snapshot index %d out of range", idx[i]);
    int rc = ensure_batch(g, nb);
    if (rc) return rc;
    NMMC_CUDA(cudaMemcpyAsync(g->d_idx, idx, sizeof(int) * nb, cudaMemcpyHostToDevice, g->stream));
    NMMC_CUDA(cudaMemcpyAsync(g->d_sig, sig, sizeof(float) * nb, cudaMemcpyHostToDevice, g->stream));
    // condition of each item from the dataset's table (device gather by a tiny copy loop)
    for (int i = 0; i < nb; ++i)
        NMMC_CUDA(cudaMemcpyAsync(g->d_cnd + 3 * i, g->cond + 3 * (size_t)idx[i], 3 * sizeof(float),
                                  cudaMemcpyDeviceToDevice, g->stream));
    const int npix = g->L * g->L;
    dim3 gi((npix + 255) / 256, nb);
    k_gen_input<<<gi, 256, 0, g->stream>>>(0, g->snaps, g->d_idx, nullptr, g->d_sig, g->d_cnd, g->L, (uint32_t)g->seed,
                                           (uint32_t)(g->seed >> 32), g->draws, g->act[0], g->target, 1.0f);
    g->draws += (unsigned long long)nb;
    if ((rc = forward(g, nb))) return rc;
    NMMC_CUDA(cudaMemsetAsync(g->d_loss, 0, sizeof(double), g->stream));
    const int np = nb * npix;
    k_gen_head<<<(np + 255) / 256, 256, 0, g->stream>>>(g->vout, g->target, np, 1.0f / (float)np, g->gv, g->d_loss);
    if ((rc = backward(g, nb))) return rc;
    if (lr > 0) {
        g->adam_t++;
        const float b1 = 0.9f, b2 = 0.999f;
        const float c1 = 1.0f - powf(b1, (float)g->adam_t), c2 = 1.0f - powf(b2, (float)g->adam_t);
        for (int l = 0; l < kGenLayers; ++l) {
            GenLayer& y = g->layer[l];
            const int n = (int)y.nw();
            k_gen_adam<<<(n + 255) / 256, 256, 0, g->stream>>>(y.w, y.gw, y.mw, y.vw, n, lr, b1, b2, c1, c2, 1e-8f);
            k_gen_adam<<<1, 64, 0, g->stream>>>(y.b, y.gb, y.mb, y.vb, y.cout, lr, b1, b2, c1, c2, 1e-8f);
        }
        if ((rc = refresh_weights(g))) return rc;
    }
    double l = 0;
    NMMC_CUDA(cudaMemcpyAsync(&l, g->d_loss, sizeof(double), cudaMemcpyDeviceToHost, g->stream));
    NMMC_CUDA(cudaStreamSynchronize(g->stream));
    if ((rc = check_flag(g))) return rc;
    if (loss) *loss = l;
    return NMMC_OK;
}

// Gradients of the last train step (lr <= 0 keeps them for inspection), parameter order.
int nmmc_gen_get_grads(nmmc_gen* g, float* out, int n) {
    if (!g || !out || n != nmmc_gen_param_count(g)) return set_error(NMMC_ERR_ARG, "bad parameter buffer");
    NMMC_CUDA(cudaStreamSynchronize(g->stream));
    size_t o = 0;
    for (int l = 0; l < kGenLayers; ++l) {
        GenLayer& y = g->layer[l];
        NMMC_CUDA(cudaMemcpy(out + o, y.gw, y.nw() * sizeof(float), cudaMemcpyDeviceToHost));
        o += y.nw();
        NMMC_CUDA(cudaMemcpy(out + o, y.gb, y.cout * sizeof(float), cudaMemcpyDeviceToHost));
        o += y.cout;
    }
    return NMMC_OK;
}

// Network input of the last step (BF16 values as float), [nb][L][L][8], for checks.
int nmmc_gen_get_input(nmmc_gen* g, int nb, float* out) {
    if (!g || !out || nb <= 0 || nb > g->bcap) return set_error(NMMC_ERR_ARG, "bad argument");
    const size_t n = (size_t)nb * g->L * g->L * kGenCin0;
    std::vector<__nv_bfloat16> h(n);
    NMMC_CUDA(cudaStreamSynchronize(g->stream));
    NMMC_CUDA(cudaMemcpy(h.data(), g->act[0], n * sizeof(__nv_bfloat16), cudaMemcpyDeviceToHost));
    for (size_t i = 0; i < n; ++i) out[i] = __bfloat162float(h[i]);
    return NMMC_OK;
}

// Warm start: for each listed chain of `ctx` (2-D Heisenberg, edge L), start from uniform
// random spins and run `steps` denoising passes at noise levels s_k = 1 - k/steps (k = 0 ..
// steps-1), re-noising the estimate to s_{k+1} between passes; the final estimate replaces
// the chain's spins. cond: (T, B, D) per chain.
int nmmc_gen_warm_start(nmmc_gen* g, nmmc_ctx* c, const int* chains, int n, const double* cond, int steps,
                        int reuse_noise) {
    if (!g || !c || !chains || !cond || n <= 0 || steps <= 0) return set_error(NMMC_ERR_ARG, "bad argument");
    if (c->dim != 2 || c->ising || c->edge != g->L || c->masked)
        return set_error(NMMC_ERR_UNSUPPORTED, "warm starts need unmasked 2-D Heisenberg lattices of edge %d", g->L);
    for (int i = 0; i < n; ++i)
        if (chains[i] < 0 || chains[i] >= c->nchains) return set_error(NMMC_ERR_ARG, "chain index out of range");
    int rc = ensure_batch(g, n);
    if (rc) return rc;
    const int npix = g->L * g->L;
    float* cur = g->target;   // the current estimate lives in the target buffer
    NMMC_CUDA(cudaMemsetAsync(cur, 0, (size_t)n * npix * kGenCout * sizeof(float), g->stream));
    std::vector<float> cf(3 * (size_t)n);
    for (size_t i = 0; i < cf.size(); ++i) cf[i] = (float)cond[i];
    NMMC_CUDA(cudaMemcpyAsync(g->d_cnd, cf.data(), cf.size() * sizeof(float), cudaMemcpyHostToDevice, g->stream));
    dim3 gi((npix + 255) / 256, n);
    // every pass's noise level goes up in one copy, so the passes run back to back with no
    // host synchronisation between them
    DeviceScratch ds;
    float* d_sigs = nullptr;
    NMMC_CUDA(ds.alloc(&d_sigs, sizeof(float) * (size_t)steps * n));
    std::vector<float> sall((size_t)steps * n);
    // noise level of pass k: linear 1 - k/steps, quadratic (1 - k/steps)^2 (more passes at low
    // noise, where the fine structure forms), or cos(pi/2 k/steps)
    const int sch = g->schedule;
    auto sched = [&](int k) -> float {
        const float f = (float)k / (float)steps;
        if (sch == 1) return (1.0f - f) * (1.0f - f);
        if (sch == 2) return cosf(1.57079632679f * f);
        return 1.0f - f;
    };
    for (int k = 0; k < steps; ++k)
        for (int i = 0; i < n; ++i) sall[(size_t)k * n + i] = sched(k);
    NMMC_CUDA(cudaMemcpyAsync(d_sigs, sall.data(), sizeof(float) * sall.size(), cudaMemcpyHostToDevice, g->stream));
    float s_prev = 1.0f;
    for (int k = 0; k < steps; ++k) {
        const float s = sched(k);
        k_gen_input<<<gi, 256, 0, g->stream>>>(reuse_noise == 2 ? 3 : (reuse_noise ? 2 : 1), nullptr, nullptr, cur,
                                               d_sigs + (size_t)k * n, g->d_cnd, g->L,
                                               (uint32_t)g->seed, (uint32_t)(g->seed >> 32), g->draws, g->act[0],
                                               nullptr, k == 0 ? 1.0f : s_prev);
        s_prev = s;
        g->draws += (unsigned long long)n;
        if ((rc = forward(g, n))) return rc;
        k_gen_normalise<<<(n * npix + 255) / 256, 256, 0, g->stream>>>(g->vout, n * npix, cur);
    }
    int* d_ch = nullptr;
    NMMC_CUDA(ds.alloc(&d_ch, sizeof(int) * n));
    NMMC_CUDA(cudaMemcpy(d_ch, chains, sizeof(int) * n, cudaMemcpyHostToDevice));
    NMMC_CUDA(cudaStreamSynchronize(c->stream));
    k_gen_to_chain<<<gi, 256, 0, g->stream>>>(c->m, (float*)c->d_spins, d_ch, cur);
    rc = cuda_check(cudaStreamSynchronize(g->stream), "k_gen_to_chain");
    return rc ? rc : check_flag(g);
}

// One layer's convolution of caller data, for checks: layer 0 (8 -> 48 channels), 1..6
// (48 -> 48) or 7 (48 -> 4); in [nimg][L][L][cin] (rounded to BF16 here), out
// [nimg][L][L][cout] FP32 = conv + bias, no activation; tensor != 0 runs the layer as the
// generator does on the tensor cores (the first and last layers only at L = 128, the FMA
// pipes otherwise), 0 on the FP32 FMA pipes.
int nmmc_gen_probe_conv(nmmc_gen* g, int layer, int nimg, const float* in, float* out, int tensor) {
    if (!g || !in || !out || layer < 0 || layer > kGenLayers - 1 || nimg <= 0) return set_error(NMMC_ERR_ARG, "bad argument");
    const int cin = layer == 0 ? kGenCin0 : kGenC, cout = layer == kGenLayers - 1 ? kGenCout : kGenC;
    const size_t LL = (size_t)g->L * g->L, ni = (size_t)nimg * LL * cin, no = (size_t)nimg * LL * cout;
    std::vector<__nv_bfloat16> h(ni);   // [img][pixel][cin] -> chunk-planar
    for (size_t i = 0; i < ni; ++i) {
        const size_t img = i / (LL * cin), r = i - img * LL * cin, pp = r / cin;
        h[pl_off<__nv_bfloat16>(cin, LL, img, pp, (int)(r - pp * cin))] = __float2bfloat16(in[i]);
    }
    DeviceScratch ds;
    __nv_bfloat16* d_in = nullptr;
    float* d_out = nullptr;
    NMMC_CUDA(cudaStreamSynchronize(g->stream));
    NMMC_CUDA(ds.alloc(&d_in, ni * sizeof(__nv_bfloat16)));
    NMMC_CUDA(ds.alloc(&d_out, no * sizeof(float)));
    int rc = cuda_check(cudaMemcpy(d_in, h.data(), ni * sizeof(__nv_bfloat16), cudaMemcpyHostToDevice), "probe H2D");
    const GenLayer& y = g->layer[layer];
    const bool tc_edge = tensor && edge_layers_on_tc(g);
    if (rc) {
    } else if (layer == 0) {
        rc = tc_edge ? conv_tma_launch<1, 1, 2, kGenC>(g, d_in, y.wb, y.b, nullptr, d_out, nimg, y.wimg)
                     : conv_launch<kGenCin0, kGenC, __nv_bfloat16, 1>(g, d_in, y.wb, y.b, nullptr, 0, d_out, nimg);
    } else if (layer == kGenLayers - 1) {
        rc = tc_edge ? conv_tma_launch<3, 6, 6, kGenCout>(g, d_in, y.wb, y.b, nullptr, d_out, nimg, y.wimg)
                     : conv_launch<kGenC, kGenCout, __nv_bfloat16, 1>(g, d_in, y.wb, y.b, nullptr, 0, d_out, nimg);
    } else {
        rc = tensor ? conv_tc_launch<1>(g, d_in, y.wb, y.b, nullptr, d_out, nimg, y.wimg)
                    : conv_launch<kGenC, kGenC, __nv_bfloat16, 1>(g, d_in, y.wb, y.b, nullptr, 0, d_out, nimg);
    }
    if (!rc) rc = cuda_check(cudaStreamSynchronize(g->stream), "probe conv");
    if (!rc) rc = check_flag(g);
    std::vector<float> ho(rc ? 0 : no);
    if (!rc) rc = cuda_check(cudaMemcpy(ho.data(), d_out, no * sizeof(float), cudaMemcpyDeviceToHost), "probe D2H");
    if (!rc)
        for (size_t i = 0; i < no; ++i) {   // chunk-planar -> [img][pixel][cout]
            const size_t img = i / (LL * cout), r = i - img * LL * cout, pp = r / cout;
            out[i] = ho[pl_off<float>(cout, LL, img, pp, (int)(r - pp * cout))];
        }
    return rc;
}

int nmmc_gen_probe_wgrad(nmmc_gen* g, int nimg, const float* in, const float* dout, float* gw, int tensor) {
    if (!g || !in || !dout || !gw || nimg <= 0) return set_error(NMMC_ERR_ARG, "bad argument");
    if (nimg > g->bcap) {
        if (int rc = ensure_batch(g, nimg)) return rc;
    }
    const int C = kGenC;
    const size_t LL = (size_t)g->L * g->L, ne = (size_t)nimg * LL * C;
    std::vector<__nv_bfloat16> hi(ne);
    std::vector<float> hg(ne);
    for (size_t i = 0; i < ne; ++i) {   // [img][pixel][c] -> chunk-planar
        const size_t img = i / (LL * C), r = i - img * LL * C, pp = r / C;
        hi[pl_off<__nv_bfloat16>(C, LL, img, pp, (int)(r - pp * C))] = __float2bfloat16(in[i]);
        hg[pl_off<float>(C, LL, img, pp, (int)(r - pp * C))] = dout[i];
    }
    DeviceScratch ds;
    __nv_bfloat16* d_in = nullptr;
    float *d_g = nullptr, *d_w = nullptr;
    NMMC_CUDA(cudaStreamSynchronize(g->stream));
    NMMC_CUDA(ds.alloc(&d_in, ne * sizeof(__nv_bfloat16)));
    NMMC_CUDA(ds.alloc(&d_g, ne * sizeof(float)));
    NMMC_CUDA(ds.alloc(&d_w, (size_t)9 * C * C * sizeof(float)));
    int rc = cuda_check(cudaMemcpy(d_in, hi.data(), ne * sizeof(__nv_bfloat16), cudaMemcpyHostToDevice), "probe H2D");
    if (!rc) rc = cuda_check(cudaMemcpy(d_g, hg.data(), ne * sizeof(float), cudaMemcpyHostToDevice), "probe H2D");
    const int keep = g->use_tc;
    g->use_tc = tensor ? 1 : 0;
    if (!rc) rc = wgrad_launch<kGenC, kGenC>(g, d_in, d_g, d_w, nimg);
    g->use_tc = keep;
    if (!rc) rc = cuda_check(cudaStreamSynchronize(g->stream), "probe wgrad");
    if (!rc) rc = check_flag(g);
    if (!rc) rc = cuda_check(cudaMemcpy(gw, d_w, (size_t)9 * C * C * sizeof(float), cudaMemcpyDeviceToHost), "probe D2H");
    return rc;
}

int nmmc_gen_set_option(nmmc_gen* g, int key, int64_t v) {
    if (!g) return set_error(NMMC_ERR_ARG, "null generator");
    if (key == NMMC_GEN_OPT_TENSOR_CORES) {
        if (v < 0 || v > 4) return set_error(NMMC_ERR_ARG, "tensor-core option must be 0 .. 4");
        NMMC_CUDA(cudaStreamSynchronize(g->stream));
        g->use_tc = v ? 1 : 0;
        g->use_ws = (v == 2) ? 1 : 0;
        g->use_tma = (v == 3) ? 0 : ((v == 4) ? 2 : 1);
        return NMMC_OK;
    }
    if (key == NMMC_GEN_OPT_SCHEDULE) {
        if (v < 0 || v > 2) return set_error(NMMC_ERR_ARG, "schedule must be 0, 1 or 2");
        g->schedule = (int)v;
        return NMMC_OK;
    }
    if (key == NMMC_GEN_OPT_WEIGHT_IMAGE) {
        if (v != 0 && v != 1) return set_error(NMMC_ERR_ARG, "weight image must be 0 or 1");
        NMMC_CUDA(cudaStreamSynchronize(g->stream));
        g->use_wimg = (int)v;
        return NMMC_OK;
    }
    if (key == NMMC_GEN_OPT_TILE_ROWS) {
        if (v != 1 && v != 2) return set_error(NMMC_ERR_ARG, "tile rows must be 1 or 2");
        NMMC_CUDA(cudaStreamSynchronize(g->stream));
        g->tile_rows = (int)v;
        return NMMC_OK;
    }
    return set_error(NMMC_ERR_ARG, "unknown generator option %d", key);
}

int nmmc_gen_save(nmmc_gen* g, const char* path) {
    if (!g || !path) return set_error(NMMC_ERR_ARG, "bad argument");
    const int n = nmmc_gen_param_count(g);
    std::vector<float> p(n);
    int rc = nmmc_gen_get_params(g, p.data(), n);
    if (rc) return rc;
    FILE* f = fopen(path, "wb");
    if (!f) return set_error(NMMC_ERR_IO, "cannot write %s", path);
    const int hdr[4] = {0x4e4d4d47, g->L, kGenLayers, n};
    bool ok = fwrite(hdr, sizeof hdr, 1, f) == 1 && fwrite(p.data(), sizeof(float), n, f) == (size_t)n;
    ok = (fclose(f) == 0) && ok;
    return ok ? NMMC_OK : set_error(NMMC_ERR_IO, "short write to %s", path);
}

int nmmc_gen_load(nmmc_gen* g, const char* path) {
    if (!g || !path) return set_error(NMMC_ERR_ARG, "bad argument");
    FILE* f = fopen(path, "rb");
    if (!f) return set_error(NMMC_ERR_IO, "cannot read %s", path);
    int hdr[4];
    const int n = nmmc_gen_param_count(g);
    std::vector<float> p(n);
    bool ok = fread(hdr, sizeof hdr, 1, f) == 1 && hdr[0] == 0x4e4d4d47 && hdr[2] == kGenLayers && hdr[3] == n &&
              fread(p.data(), sizeof(float), n, f) == (size_t)n;
    fclose(f);
    if (!ok) return set_error(NMMC_ERR_IO, "%s is not a generator of this shape", path);
    return nmmc_gen_set_params(g, p.data(), n);
}

}  // extern "C"
