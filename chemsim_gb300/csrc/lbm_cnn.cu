// lbm_cnn.cu — the coarse-grid correction network and the kernels around it.
//
// No reference counterpart: a learned correction for a 4x-coarsened lattice.
// The network is 4 layers of 3x3 convolutions, channels 4 -> 32 -> 32 -> 32
// -> 9, GELU (tanh form) between layers, bf16 weights and activations, f32
// accumulation.
//
// Activation layout ("CB8"): [image][row + 1][channel block][x + 1][8] bf16,
// i.e. blocks of 8 channels, a one-pixel zero halo around the image.  A run of
// 8 pixels x 8 channels is then 128 contiguous bytes — exactly one UMMA core
// matrix — so for a 3x3 convolution as an implicit GEMM (M = pixels, N =
// output channels, K = 9 taps x input channels) the A operand of every tap is
// a shared-memory descriptor pointing into one staged halo tile, offset by the
// tap: no im2col copy.  The B operand (weights) is pre-packed into the same
// core-matrix layout.  One CTA = 128 pixels of one row; one thread issues the
// 9 x Cin/16 tcgen05.mma into a TMEM accumulator (128 lanes x N f32 columns);
// the 4 warps read their 32 lanes back with tcgen05.ld and run the epilogue
// (bias, GELU, stores).  The same kernel computes input gradients with the
// flipped, channel-transposed weights and a GELU' epilogue.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "lbm_cb8.cuh"
#include "lbm_handle.cuh"
#include "lbm_tc.cuh"

using namespace lbmk;

namespace {

constexpr int kLayers = 4;
constexpr int kCin[kLayers] = {4, 32, 32, 32};
constexpr int kCout[kLayers] = {32, 32, 32, 9};
constexpr int kTileM = 128;                       // pixels per CTA
constexpr uint32_t kWaitPolls = 1u << 22;         // bounded mbarrier wait
constexpr char kCnnMagic[8] = {'L', 'B', 'M', 'C', 'N', 'N', '0', '1'};

__host__ __device__ constexpr int pad16(int c) { return (c + 15) / 16 * 16; }

// GELU (erf form) and its derivative.
// GELU in its tanh form, 0.5 x (1 + tanh(sqrt(2/pi) (x + 0.044715 x^3)))
// (Hendrycks & Gimpel), with the hardware tanh.approx: a few FMAs and one
// MUFU op per value, where the erf form costs tens of instructions and made
// the convolution epilogue issue-bound.
__device__ __forceinline__ float tanh_fast(float x) {
    float y;
    asm("tanh.approx.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}
constexpr float kGeluK = 0.7978845608028654f;     // sqrt(2 / pi)
constexpr float kGeluC = 0.044715f;
__device__ __forceinline__ float gelu(float x) {
    const float t = tanh_fast(kGeluK * fmaf(kGeluC * x, x * x, x));
    return 0.5f * x * (1.0f + t);
}
__device__ __forceinline__ float gelu_grad(float x) {
    const float t = tanh_fast(kGeluK * fmaf(kGeluC * x, x * x, x));
    const float du = kGeluK * fmaf(3.0f * kGeluC, x * x, 1.0f);
    return 0.5f * (1.0f + t) + 0.5f * x * (1.0f - t * t) * du;
}

struct ConvArgs {
    const __nv_bfloat16* in;      // CB8, CBI blocks
    const __nv_bfloat16* wpack;   // packed B operand
    const float* bias;            // NO (forward) or null
    __nv_bfloat16* z_out;         // CB8, NO/8 blocks (mode 0)
    __nv_bfloat16* x_out;         // CB8, NO/8 blocks (mode 0); gradient out (mode 2)
    float* f32_out;               // NCHW, nreal channels (mode 1)
    const __nv_bfloat16* zprev;   // CB8, NO/8 blocks (mode 2)
    int B, H, W, nreal;
    int* err;
};

// Epilogue of one 128-pixel tile (the CTA's 4 warps, lane = pixel): bias +
// GELU (MODE 0), f32 NCHW output (MODE 1), or x GELU' of the previous
// layer's pre-activation (MODE 2).
template <int NO, int MODE>
__device__ __forceinline__ void conv_epilogue(const ConvArgs& a, const float (&v)[NO], int b, int y,
                                              int x) {
    const int H = a.H, W = a.W;
    if constexpr (MODE == 0) {
#pragma unroll
        for (int cb = 0; cb < NO / 8; ++cb) {
            float z[8], gv[8];
#pragma unroll
            for (int c = 0; c < 8; ++c) {
                z[c] = v[cb * 8 + c] + a.bias[cb * 8 + c];
                gv[c] = gelu(z[c]);
            }
            const int64_t o = cb8_chunk(b, y, cb, x, H, W, NO / 8);
            if (a.z_out != nullptr) reinterpret_cast<uint4*>(a.z_out)[o] = pack8_bf16(z);
            reinterpret_cast<uint4*>(a.x_out)[o] = pack8_bf16(gv);
        }
    } else if constexpr (MODE == 1) {
        for (int c = 0; c < a.nreal; ++c)
            a.f32_out[((int64_t(b) * a.nreal + c) * H + y) * W + x] = v[c] + a.bias[c];
    } else {
#pragma unroll
        for (int cb = 0; cb < NO / 8; ++cb) {
            const int64_t o = cb8_chunk(b, y, cb, x, H, W, NO / 8);
            float zp[8], gv[8];
            unpack8_bf16(__ldg(reinterpret_cast<const uint4*>(a.zprev) + o), zp);
#pragma unroll
            for (int c = 0; c < 8; ++c) gv[c] = v[cb * 8 + c] * gelu_grad(zp[c]);
            reinterpret_cast<uint4*>(a.x_out)[o] = pack8_bf16(gv);
        }
    }
}

// Dynamic shared memory of a conv CTA: A halo tile (3 rows x CBI blocks x
// 130 pixels x 16 B; the descriptors of the 9 taps reach exactly its last
// byte), B (weights), two mbarriers and the TMEM address slot.
// Output rows per CTA, one after the other, with the weights staged and the
// accumulator allocated once.  8 x 512^2 forward / gradient call on one GB300
// (a timing loop that waits for each call): 1 row 0.450 / 1.899 ms, 2 rows
// 0.395 / 1.784, 4 rows 0.403 / 1.806.
#ifndef LBM_CONV_ROWS
#define LBM_CONV_ROWS 2
#endif
// Sized per instantiation, so layers with fewer input blocks or outputs keep
// more CTAs resident (e.g. 4 -> 32 channels: 22.6 KB, 10 CTAs per SM instead
// of 5 at the 44 KB of a 32 -> 32 layer).
constexpr int kRowBytes = (kTileM + 2) * 16;
template <int CBI>
constexpr int conv_a_region() { return (3 * CBI * kRowBytes + 1023) / 1024 * 1024; }
template <int CBI, int NO>
constexpr int conv_b_bytes() { return 9 * (CBI / 2) * (NO / 8) * 2 * 128; }
template <int CBI, int NO>
constexpr int conv_smem() { return conv_a_region<CBI>() + conv_b_bytes<CBI, NO>() + 64; }

template <int CBI, int NO, int MODE>
__global__ void __launch_bounds__(128)
conv3x3_tc_kernel(const ConvArgs a) {
    extern __shared__ __align__(1024) uint8_t smem[];
    uint8_t* sA = smem;
    constexpr int kARegion = conv_a_region<CBI>(), kBRegion = conv_b_bytes<CBI, NO>();
    uint8_t* sB = smem + kARegion;
    uint64_t* bar = reinterpret_cast<uint64_t*>(smem + kARegion + kBRegion);   // MMAs done
    uint64_t* lbar = bar + 1;                                                  // tiles staged
    uint32_t* tslot = reinterpret_cast<uint32_t*>(smem + kARegion + kBRegion + 16);
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int x0 = blockIdx.x * kTileM, y = blockIdx.y, b = blockIdx.z;
    const int H = a.H, W = a.W;
    // B: 9 * CBI/2 K-steps of (NO/8 x 2) core matrices; A: rows y-1..y+1 of
    // every input block, pixels x0-1 .. x0+128 (in the halo, so in bounds:
    // W is a multiple of 128 and the layout has one halo pixel each side)
    constexpr uint32_t kBBytes = 9 * (CBI / 2) * (NO / 8) * 2 * 128;
    constexpr uint32_t kABytes = 3 * CBI * kRowBytes;
    static_assert(kBBytes <= kBRegion && kABytes <= kARegion, "tiles fit");

    if (tid == 0) {
        lbmtc::mbar_init(bar, 1);
        lbmtc::mbar_init(lbar, 1);
    }
    if (warp == 0) lbmtc::tmem_alloc(tslot, 32);
    __syncthreads();
    // LBM_CONV_ROWS output rows of one 128-pixel column per CTA, one after the
    // other: the weights are staged and the accumulator allocated once; each
    // row restages its 3 input rows.  Each barrier completes once per row, so
    // row r waits on phase r & 1.
    uint32_t tmem = 0;
    const int y_first = y * LBM_CONV_ROWS;
#pragma unroll 1
    for (int r = 0; r < LBM_CONV_ROWS; ++r) {
        const int yr = y_first + r;
        if (yr >= H) break;                     // CTA-uniform
        const uint32_t phase = uint32_t(r) & 1u;
        if (tid == 0) {
            // stage with the bulk-copy engine: one copy of the packed weights
            // (first row only) and one contiguous 2080-byte row segment per
            // (row, input block)
            lbmtc::mbar_expect_tx(lbar, (r == 0 ? kBBytes : 0u) + kABytes);
            if (r == 0) lbmtc::bulk_g2s(sB, a.wpack, kBBytes, lbar);
            const uint4* in = reinterpret_cast<const uint4*>(a.in);
#pragma unroll
            for (int rr = 0; rr < 3; ++rr)
#pragma unroll
                for (int cb = 0; cb < CBI; ++cb)
                    lbmtc::bulk_g2s(sA + (rr * CBI + cb) * kRowBytes,
                                    in + cb8_chunk(b, yr + rr - 1, cb, x0 - 1, H, W, CBI), kRowBytes, lbar);
        }
        bool mine = lbmtc::mbar_wait_bounded(lbar, phase, kWaitPolls);
        if (!mine) {
            if (lane == 0) atomicExch(a.err, 1);
            (void)lbmtc::mbar_wait_bounded(lbar, phase, kWaitPolls);   // let the copies land
        }
        lbmtc::fence_before_sync();             // orders the TMEM allocation / last reads before the barrier
        const bool staged = __syncthreads_and(mine);
        lbmtc::fence_after_sync();
        tmem = *tslot;

        if (tid == 0 && staged) {
            constexpr uint32_t idesc = lbmtc::idesc_bf16_f32(kTileM, NO);
            const uint32_t a0 = lbmtc::smem_u32(sA), b0 = lbmtc::smem_u32(sB);
            uint32_t acc = 0;
#pragma unroll 1
            for (int t = 0; t < 9; ++t) {
                const int ky = t / 3, kx = t % 3;
#pragma unroll
                for (int j = 0; j < CBI / 2; ++j) {
                    // A: core (m, k) of this step at ((ky*CBI + 2j + k) * 130 + kx + 8m) * 16
                    const uint32_t aaddr = a0 + uint32_t(((ky * CBI + 2 * j) * (kTileM + 2) + kx) * 16);
                    const uint64_t ad = lbmtc::smem_desc(aaddr, (kTileM + 2) * 16, 128);
                    // B: core (n, k) of step s at s * (NO/8 * 2 * 128) + (n * 2 + k) * 128
                    const uint32_t baddr = b0 + uint32_t((t * (CBI / 2) + j) * (NO / 8) * 2 * 128);
                    const uint64_t bd = lbmtc::smem_desc(baddr, 128, 256);
                    lbmtc::mma_bf16(tmem, ad, bd, idesc, acc);
                    acc = 1;
                }
            }
            lbmtc::mma_commit(bar);
        }
        bool done = staged && lbmtc::mbar_wait_bounded(bar, phase, kWaitPolls);
        if (staged && !done) {
            if (lane == 0) atomicExch(a.err, 1);
            (void)lbmtc::mbar_wait_bounded(bar, phase, kWaitPolls);   // let the MMAs drain
        }
        lbmtc::fence_after_sync();

        float v[NO];
        const uint32_t taddr = tmem + (uint32_t(warp * 32) << 16);
        if constexpr (NO == 32) lbmtc::tmem_ld32(taddr, v);
        else lbmtc::tmem_ld16(taddr, v);

        const int x = x0 + warp * 32 + lane;
        if (done && x < W) conv_epilogue<NO, MODE>(a, v, b, yr, x);
        // every warp has read the accumulator, and the MMAs no longer read
        // the staged rows, before the next row overwrites either
        lbmtc::fence_before_sync();
        const bool go_on = __syncthreads_and(done);
        lbmtc::fence_after_sync();
        if (!go_on) break;                      // CTA-uniform
    }
    tmem = *tslot;
    if (warp == 0) lbmtc::tmem_dealloc(tmem, 32);
}

// W f32 [9][cin][cout] -> the conv kernel's B image for a forward layer
// (K = taps x input channels padded to 16, N = outputs padded to NO).
__global__ void pack_fwd_kernel(const float* __restrict__ Wt, int cin, int cout, int cbi, int no,
                                __nv_bfloat16* __restrict__ out) {
    const int total = 9 * (cbi / 2) * (no / 8) * 2 * 64;
    for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < total; e += gridDim.x * blockDim.x) {
        const int c = e & 7, r = (e >> 3) & 7;
        int q = e >> 6;                         // core index within everything
        const int kc = q & 1;
        q >>= 1;
        const int nc = q % (no / 8);
        const int s = q / (no / 8);
        const int j = s % (cbi / 2), t = s / (cbi / 2);
        const int ci = 8 * (2 * j + kc) + c, co = 8 * nc + r;
        const float w = (ci < cin && co < cout) ? Wt[(t * cin + ci) * cout + co] : 0.f;
        out[e] = __float2bfloat16_rn(w);
    }
}

// The B image of the input-gradient convolution of a layer: input = the
// layer's output gradient (cout channels), output = cin channels, weights
// W'[t][co][ci] = W[8 - t][ci][co] (taps flipped).
__global__ void pack_dx_kernel(const float* __restrict__ Wt, int cin, int cout, int cbi, int no,
                               __nv_bfloat16* __restrict__ out) {
    const int total = 9 * (cbi / 2) * (no / 8) * 2 * 64;
    for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < total; e += gridDim.x * blockDim.x) {
        const int c = e & 7, r = (e >> 3) & 7;
        int q = e >> 6;
        const int kc = q & 1;
        q >>= 1;
        const int nc = q % (no / 8);
        const int s = q / (no / 8);
        const int j = s % (cbi / 2), t = s / (cbi / 2);
        const int co = 8 * (2 * j + kc) + c, ci = 8 * nc + r;
        const float w = (ci < cin && co < cout) ? Wt[((8 - t) * cin + ci) * cout + co] : 0.f;
        out[e] = __float2bfloat16_rn(w);
    }
}

// NCHW f32 (C channels) -> CB8 bf16 (CB blocks, extra channels zero).
__global__ void nchw_to_cb8_kernel(const float* __restrict__ in, int B, int C, int H, int W, int CB,
                                   __nv_bfloat16* __restrict__ out) {
    const int64_t n = int64_t(B) * H * W * CB;
    for (int64_t e = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; e < n;
         e += int64_t(gridDim.x) * blockDim.x) {
        const int x = int(e % W);
        int64_t q = e / W;
        const int y = int(q % H);
        q /= H;
        const int cb = int(q % CB);
        const int b = int(q / CB);
        float v[8];
#pragma unroll
        for (int c = 0; c < 8; ++c) {
            const int ch = cb * 8 + c;
            v[c] = ch < C ? in[((int64_t(b) * C + ch) * H + y) * W + x] : 0.f;
        }
        reinterpret_cast<uint4*>(out)[cb8_chunk(b, y, cb, x, H, W, CB)] = pack8_bf16(v);
    }
}

// MSE loss over all outputs; writes the loss gradient (CB8 bf16, 2 blocks)
// and per-block partial sums of the squared error.
__global__ void __launch_bounds__(256)
mse_kernel(const float* __restrict__ out, const float* __restrict__ target, int B, int C, int H,
           int W, float grad_scale, __nv_bfloat16* __restrict__ g, double* __restrict__ partial) {
    const int64_t n = int64_t(B) * H * W;
    double acc = 0.0;
    for (int64_t e = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; e < n;
         e += int64_t(gridDim.x) * blockDim.x) {
        const int x = int(e % W);
        const int y = int((e / W) % H);
        const int b = int(e / (int64_t(W) * H));
        float gv[16];
#pragma unroll
        for (int c = 0; c < 16; ++c) gv[c] = 0.f;
        for (int c = 0; c < C; ++c) {
            const int64_t o = ((int64_t(b) * C + c) * H + y) * W + x;
            const float d = out[o] - target[o];
            acc += double(d) * double(d);
            gv[c] = grad_scale * d;
        }
        reinterpret_cast<uint4*>(g)[cb8_chunk(b, y, 0, x, H, W, 2)] = pack8_bf16(gv);
        reinterpret_cast<uint4*>(g)[cb8_chunk(b, y, 1, x, H, W, 2)] = pack8_bf16(gv + 8);
    }
    __shared__ double s[256];
    s[threadIdx.x] = acc;
    __syncthreads();
    for (int k = 128; k > 0; k >>= 1) {
        if (threadIdx.x < k) s[threadIdx.x] += s[threadIdx.x + k];
        __syncthreads();
    }
    if (threadIdx.x == 0) partial[blockIdx.x] = s[0];
}

// Weight gradient of one layer on the CUDA cores, partial per block:
// dW[t][ci][co] += sum_pixels x[p + off(t)][ci] * g[p][co].  One thread per
// (tap, input channel), all output channels in registers; a block walks
// 128-pixel row segments; the x halo tile (bf16, as stored) and the g
// segment (f32) are staged in shared memory.
template <int CIN_B, int COUT_B>
__global__ void __launch_bounds__(288)
dw_partial_kernel(const __nv_bfloat16* __restrict__ x, const __nv_bfloat16* __restrict__ g, int B,
                  int H, int W, int cin, int cout, float* __restrict__ partial,
                  float* __restrict__ bias_partial) {
    constexpr int CO = COUT_B * 8;
    __shared__ __nv_bfloat16 sx[3][CIN_B * 8][kTileM + 2];     // <= 25 KB
    __shared__ float sg[kTileM][CO];                            // <= 16 KB
    const int tid = threadIdx.x;
    const int pairs = 9 * cin;
    const int t = tid / cin, ci = tid - t * cin;
    float acc[CO];
#pragma unroll
    for (int c = 0; c < CO; ++c) acc[c] = 0.f;
    float bacc = 0.f;                              // bias gradient: thread co < cout
    const int segs_per_row = (W + kTileM - 1) / kTileM;
    const int64_t nseg = int64_t(B) * H * segs_per_row;
    for (int64_t sgi = blockIdx.x; sgi < nseg; sgi += gridDim.x) {
        const int sx0 = int(sgi % segs_per_row) * kTileM;
        const int y = int((sgi / segs_per_row) % H);
        const int b = int(sgi / (int64_t(segs_per_row) * H));
        __syncthreads();
        for (int k = tid; k < 3 * CIN_B * (kTileM + 2); k += blockDim.x) {
            const int px = k % (kTileM + 2);
            const int rc = k / (kTileM + 2);
            const int cb = rc % CIN_B, r = rc / CIN_B;
            float v[8];
            const int xx = sx0 + px - 1;
            if (xx < W)
                unpack8_bf16(__ldg(reinterpret_cast<const uint4*>(x) + cb8_chunk(b, y + r - 1, cb, xx, H, W, CIN_B)), v);
            else
                for (int c = 0; c < 8; ++c) v[c] = 0.f;
            for (int c = 0; c < 8; ++c) sx[r][cb * 8 + c][px] = __float2bfloat16_rn(v[c]);
        }
        for (int k = tid; k < kTileM * COUT_B; k += blockDim.x) {
            const int px = k % kTileM, cb = k / kTileM;
            float v[8];
            const int xx = sx0 + px;
            if (xx < W)
                unpack8_bf16(__ldg(reinterpret_cast<const uint4*>(g) + cb8_chunk(b, y, cb, xx, H, W, COUT_B)), v);
            else
                for (int c = 0; c < 8; ++c) v[c] = 0.f;
            for (int c = 0; c < 8; ++c) sg[px][cb * 8 + c] = v[c];
        }
        __syncthreads();
        if (tid < pairs) {
            const int ky = t / 3, kx = t % 3;
            for (int p = 0; p < kTileM; ++p) {
                const float xv = __bfloat162float(sx[ky][ci][p + kx]);
#pragma unroll
                for (int c = 0; c < CO; ++c) acc[c] = fmaf(xv, sg[p][c], acc[c]);
            }
        }
        if (tid < cout)
            for (int p = 0; p < kTileM; ++p) bacc += sg[p][tid];
    }
    if (tid < pairs) {
        float* dst = partial + (int64_t(blockIdx.x) * pairs + tid) * cout;
        for (int c = 0; c < cout; ++c) dst[c] = acc[c];
    }
    if (tid < cout) bias_partial[int64_t(blockIdx.x) * cout + tid] = bacc;
}

// Weight and bias gradients of one layer on the tensor cores, partial per
// CTA: an implicit GEMM with the pixels as the reduction dimension,
//   D[(t, ci)][co] = sum_p x[p + off(t)][ci] g[p][co],
// M = (tap, input channel) rows, N = output channels, K = pixels.  Both
// operands are read from the CB8 layout as stored: there a pixel's 8
// channels are 16 contiguous bytes, so a run of 8 pixels of one channel
// block is a core matrix with the channels along M (or N) — the MN-major
// form of the UMMA operands, no transposition.  Per 128-pixel row segment
// the CTA stages, with the bulk-copy engine, the segment's pixel run of every
// (tap, input block) (a tap's one-pixel shift is a 16-byte offset of the
// copy's source) and of every output block of g; M-tiles of 128 rows = 16
// (tap, block) runs, so 4 taps of 32 channels per MMA (8 taps of 16 for the
// first layer) and the last M-tile padded with zero runs, one of which is
// all ones: its D rows are sum_p g[p][co], the bias gradient.  The
// accumulators stay in TMEM across the CTA's segments.
constexpr int kDwRun = kTileM * 16;                      // bytes of one staged pixel run
template <int CIN_B>
constexpr int dw_groups() { return (9 * CIN_B + 1 + 15) / 16; }   // M-tiles (with the ones run)


template <int CIN_B, int COUT_B>
__global__ void __launch_bounds__(128)
dw_tc_kernel(const __nv_bfloat16* __restrict__ x, const __nv_bfloat16* __restrict__ g, int B,
             int H, int W, int cin, int cout, float* __restrict__ partial,
             float* __restrict__ bias_partial, int* __restrict__ err) {
    constexpr int G = dw_groups<CIN_B>();
    constexpr int NRUNS = 16 * G;                  // A runs, padding included
    constexpr int N = COUT_B * 8;
    constexpr int ONES = 9 * CIN_B;                // the run of ones (first padding run)
    extern __shared__ __align__(1024) uint8_t smem[];
    uint8_t* sA = smem;
    uint8_t* sB = smem + NRUNS * kDwRun;
    uint64_t* lbar = reinterpret_cast<uint64_t*>(sB + COUT_B * kDwRun);
    uint64_t* mbar = lbar + 1;
    uint32_t* tslot = reinterpret_cast<uint32_t*>(lbar + 2);
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;

    // padding runs: zeros, the first of them ones (bf16 1.0 = 0x3F80)
    for (int k = tid; k < (NRUNS - ONES) * kDwRun / 16; k += blockDim.x) {
        const int run = ONES + k / (kDwRun / 16);
        const uint32_t v = run == ONES ? 0x3F803F80u : 0u;
        reinterpret_cast<uint4*>(sA + ONES * kDwRun)[k] = make_uint4(v, v, v, v);
    }
    lbmtc::fence_proxy_async_smem();
    if (tid == 0) {
        lbmtc::mbar_init(lbar, 1);
        lbmtc::mbar_init(mbar, 1);
    }
    if (warp == 0) lbmtc::tmem_alloc(tslot, 128);
    lbmtc::fence_before_sync();
    __syncthreads();
    lbmtc::fence_after_sync();
    const uint32_t tmem = *tslot;

    // MN-major operands, no swizzle: core matrices of 128 bytes (8 pixels x
    // 8 channels); the leading byte offset is the step between core matrices
    // along K (pixels, 128 bytes), the stride byte offset the step along M / N
    // (one run).  (Checked against the oracle's gradients; the two offsets
    // the other way round give wrong sums.)
    constexpr uint32_t lbo = 128, sbo = kDwRun;
    constexpr uint32_t idesc = lbmtc::idesc_bf16_f32(128, N) | (1u << 15) | (1u << 16);
    const uint32_t a0 = lbmtc::smem_u32(sA), b0 = lbmtc::smem_u32(sB);

    const int segs_per_row = W / kTileM;
    const int64_t nseg = int64_t(B) * H * segs_per_row;
    uint32_t phase = 0, acc = 0;
    bool ok = true;
    const uint4* xin = reinterpret_cast<const uint4*>(x);
    const uint4* gin = reinterpret_cast<const uint4*>(g);
    for (int64_t sgi = blockIdx.x; sgi < nseg && ok; sgi += gridDim.x) {
        const int x0 = int(sgi % segs_per_row) * kTileM;
        const int y = int((sgi / segs_per_row) % H);
        const int b = int(sgi / (int64_t(segs_per_row) * H));
        if (tid == 0) {
            lbmtc::mbar_expect_tx(lbar, (9 * CIN_B + COUT_B) * kDwRun);
#pragma unroll 1
            for (int t = 0; t < 9; ++t) {
                const int ky = t / 3, kx = t % 3;
                for (int cb = 0; cb < CIN_B; ++cb)
                    lbmtc::bulk_g2s(sA + (t * CIN_B + cb) * kDwRun,
                                    xin + cb8_chunk(b, y + ky - 1, cb, x0 + kx - 1, H, W, CIN_B),
                                    kDwRun, lbar);
            }
            for (int cb = 0; cb < COUT_B; ++cb)
                lbmtc::bulk_g2s(sB + cb * kDwRun, gin + cb8_chunk(b, y, cb, x0, H, W, COUT_B), kDwRun,
                                lbar);
        }
        bool staged = lbmtc::mbar_wait_bounded(lbar, phase, kWaitPolls);
        if (!staged) {
            if (lane == 0) atomicExch(err, 1);
            (void)lbmtc::mbar_wait_bounded(lbar, phase, kWaitPolls);
        }
        staged = __syncthreads_and(staged);
        lbmtc::fence_after_sync();
        if (!staged) { ok = false; break; }
        if (tid == 0) {
#pragma unroll 1
            for (int s = 0; s < kTileM / 16; ++s) {
                const uint64_t bd = lbmtc::smem_desc(b0 + uint32_t(s * 256), lbo, sbo);
#pragma unroll
                for (int q = 0; q < G; ++q) {
                    const uint64_t ad = lbmtc::smem_desc(a0 + uint32_t(q * 16 * kDwRun + s * 256), lbo, sbo);
                    lbmtc::mma_bf16(tmem + uint32_t(q * N), ad, bd, idesc, acc);
                }
                acc = 1;
            }
            lbmtc::mma_commit(mbar);
        }
        // the MMAs read the staged tiles: wait for them before the next copy
        bool done = lbmtc::mbar_wait_bounded(mbar, phase, kWaitPolls);
        if (!done) {
            if (lane == 0) atomicExch(err, 1);
            (void)lbmtc::mbar_wait_bounded(mbar, phase, kWaitPolls);
        }
        ok = __syncthreads_and(done);
        lbmtc::fence_after_sync();
        phase ^= 1u;
        acc = 1;
    }

    // TMEM -> partials: lane l of warp w holds D row 32 w + l of every M-tile
    const int row = warp * 32 + lane;
#pragma unroll
    for (int q = 0; q < G; ++q) {
        float v[N];
        const uint32_t taddr = tmem + uint32_t(q * N) + (uint32_t(warp * 32) << 16);
        if constexpr (N == 32) lbmtc::tmem_ld32(taddr, v);
        else lbmtc::tmem_ld16(taddr, v);
        const int run = q * 16 + row / 8, c = row % 8;
        if (acc == 0) {
#pragma unroll
            for (int n = 0; n < N; ++n) v[n] = 0.f;      // no segment: nothing accumulated
        }
        if (run < 9 * CIN_B) {
            const int t = run / CIN_B, ci = (run % CIN_B) * 8 + c;
            if (ci < cin) {
                float* dst = partial + (int64_t(blockIdx.x) * 9 * cin + t * cin + ci) * cout;
#pragma unroll
                for (int n = 0; n < N; ++n)
                    if (n < cout) dst[n] = v[n];
            }
        } else if (run == ONES && c == 0) {
#pragma unroll
            for (int n = 0; n < N; ++n)
                if (n < cout) bias_partial[int64_t(blockIdx.x) * cout + n] = v[n];
        }
    }
    lbmtc::fence_before_sync();
    __syncthreads();
    if (warp == 0) lbmtc::tmem_dealloc(tmem, 128);
}

template <int CIN_B, int COUT_B>
constexpr int dw_smem() {
    return 16 * dw_groups<CIN_B>() * kDwRun + COUT_B * kDwRun + 64;
}

// grad[k] = sum over blocks of partial[block][k] (fixed order).
__global__ void reduce_partials_kernel(const float* __restrict__ partial, int nblocks, int n,
                                       float* __restrict__ grad) {
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x) {
        float s = 0.f;
        for (int q = 0; q < nblocks; ++q) s += partial[int64_t(q) * n + k];
        grad[k] = s;
    }
}

__global__ void adam_kernel(float* __restrict__ p, const float* __restrict__ g, float* __restrict__ m,
                            float* __restrict__ v, int n, float lr, float b1, float b2, float eps,
                            float c1, float c2) {
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x) {
        const float gk = g[k];
        const float mk = b1 * m[k] + (1.f - b1) * gk;
        const float vk = b2 * v[k] + (1.f - b2) * gk * gk;
        m[k] = mk;
        v[k] = vk;
        p[k] -= lr * (mk / c1) / (sqrtf(vk / c2) + eps);
    }
}

// One warp waits on an mbarrier that nothing signals, with the same bounded
// wait as the convolution kernels, and records that it gave up.
__global__ void wait_probe_kernel(int* __restrict__ timed_out, uint32_t polls) {
    __shared__ uint64_t bar;
    if (threadIdx.x == 0) lbmtc::mbar_init(&bar, 1);
    __syncthreads();
    const bool ok = lbmtc::mbar_wait_bounded(&bar, 0, polls);
    if (!ok && threadIdx.x == 0) atomicExch(timed_out, 1);
}

int grid_of(int64_t n, int block) {
    int64_t g = (n + block - 1) / block;
    if (g > 65535 * 4) g = 65535 * 4;
    return int(g < 1 ? 1 : g);
}

}  // namespace

// ---------------------------------------------------------------------------

struct lbm_cnn {
    int H = 0, W = 0, maxB = 0;
    int nparams = 0;
    int off_w[kLayers] = {}, off_b[kLayers] = {};
    float* params = nullptr;      // master f32 weights and biases
    float* grads = nullptr;
    float* adam_m = nullptr;
    float* adam_v = nullptr;
    int adam_t = 0;
    __nv_bfloat16* wf[kLayers] = {};   // forward B images
    __nv_bfloat16* wd[kLayers] = {};   // input-gradient B images (layers 1..3)
    __nv_bfloat16* x[kLayers] = {};    // layer inputs (x[0] = features), CB8
    __nv_bfloat16* z[kLayers] = {};    // pre-activations of layers 0..2 outputs (z[l] for layer l)
    __nv_bfloat16* gbuf[kLayers + 1] = {};  // gradients wrt layer outputs
    float* out = nullptr;              // NCHW f32, 9 channels
    float* feat = nullptr;             // one image of features (4 x H x W f32), lbm_coarse_run
    float* dw_partial = nullptr;
    float* db_partial = nullptr;
    double* loss_partial = nullptr;
    int* err = nullptr;
    int dw_blocks = 0;
    cudaStream_t stream = nullptr;     // where every call issues its work
    cudaStream_t own = nullptr;        // created with the net; used when no stream is set
    int dev = 0;
};

namespace {

int cfail(int code, const std::string& msg) { return lattice_fail(code, msg); }

#define CNN_CUDA(expr)                                                            \
    do {                                                                          \
        cudaError_t e__ = (expr);                                                 \
        if (e__ != cudaSuccess) {                                                 \
            (void)cudaGetLastError();                                             \
            return cfail(e__ == cudaErrorMemoryAllocation ? LBM_ERR_OUT_OF_MEMORY  \
                                                          : LBM_ERR_CUDA,         \
                         std::string(#expr) + ": " + cudaGetErrorString(e__));    \
        }                                                                         \
    } while (0)

int cbi_of(int c) { return pad16(c) / 8; }
size_t cb8_bytes(const lbm_cnn* N, int B, int cb) {
    return size_t(B) * (N->H + 2) * cb * (N->W + 2) * 16;
}

template <int CBI, int NO, int MODE>
cudaError_t launch_conv(const lbm_cnn* N, const ConvArgs& a) {
    static bool configured = false;
    if (!configured) {
        cudaError_t e = cudaFuncSetAttribute(conv3x3_tc_kernel<CBI, NO, MODE>,
                                             cudaFuncAttributeMaxDynamicSharedMemorySize,
                                             conv_smem<CBI, NO>());
        if (e != cudaSuccess) return e;
        configured = true;
    }
    const dim3 grid((a.W + kTileM - 1) / kTileM, (a.H + LBM_CONV_ROWS - 1) / LBM_CONV_ROWS, a.B);
    conv3x3_tc_kernel<CBI, NO, MODE><<<grid, 128, conv_smem<CBI, NO>(), N->stream>>>(a);
    return cudaGetLastError();
}

// Weight gradients on the tensor cores (1) or on the CUDA cores (0).
#ifndef LBM_DW_TC
#define LBM_DW_TC 1
#endif

template <int CIN_B, int COUT_B>
cudaError_t launch_dw(const lbm_cnn* N, const __nv_bfloat16* x, const __nv_bfloat16* g, int B,
                      int cin, int cout) {
    static bool configured = false;
    if (!configured) {
        cudaError_t e = cudaFuncSetAttribute(dw_tc_kernel<CIN_B, COUT_B>,
                                             cudaFuncAttributeMaxDynamicSharedMemorySize,
                                             dw_smem<CIN_B, COUT_B>());
        if (e != cudaSuccess) return e;
        configured = true;
    }
    dw_tc_kernel<CIN_B, COUT_B><<<N->dw_blocks, 128, dw_smem<CIN_B, COUT_B>(), N->stream>>>(
        x, g, B, N->H, N->W, cin, cout, N->dw_partial, N->db_partial, N->err);
    return cudaGetLastError();
}

int repack(lbm_cnn* N) {
    for (int l = 0; l < kLayers; ++l) {
        const int cbi = cbi_of(kCin[l]), no = pad16(kCout[l]);
        pack_fwd_kernel<<<64, 256, 0, N->stream>>>(N->params + N->off_w[l], kCin[l], kCout[l], cbi, no,
                                                   N->wf[l]);
        CNN_CUDA(cudaGetLastError());
        if (l > 0) {
            const int cbi_d = cbi_of(kCout[l]), no_d = pad16(kCin[l]);
            pack_dx_kernel<<<64, 256, 0, N->stream>>>(N->params + N->off_w[l], kCin[l], kCout[l],
                                                      cbi_d, no_d, N->wd[l]);
            CNN_CUDA(cudaGetLastError());
        }
    }
    return LBM_OK;
}

// Forward pass over B images whose features are in N->x[0].
// Pre-activations are stored only for training (the backward pass needs
// them); inference skips those writes.
int forward_impl(lbm_cnn* N, int B, bool keep_z) {
    for (int l = 0; l < kLayers; ++l) {
        ConvArgs a{};
        a.in = N->x[l];
        a.wpack = N->wf[l];
        a.bias = N->params + N->off_b[l];
        a.B = B;
        a.H = N->H;
        a.W = N->W;
        a.err = N->err;
        cudaError_t e;
        if (l < kLayers - 1) {
            a.z_out = keep_z ? N->z[l] : nullptr;
            a.x_out = N->x[l + 1];
            e = (l == 0) ? launch_conv<2, 32, 0>(N, a) : launch_conv<4, 32, 0>(N, a);
        } else {
            a.f32_out = N->out;
            a.nreal = kCout[l];
            e = launch_conv<4, 16, 1>(N, a);
        }
        if (e != cudaSuccess) { (void)cudaGetLastError(); return cfail(LBM_ERR_CUDA, cudaGetErrorString(e)); }
    }
    return LBM_OK;
}

// Backward pass given the loss gradient in N->gbuf[kLayers] (CB8, 2 blocks):
// weight / bias gradients into N->grads.
int backward_impl(lbm_cnn* N, int B) {
    for (int l = kLayers - 1; l >= 0; --l) {
        const __nv_bfloat16* g = N->gbuf[l + 1];
        // weight and bias gradient of layer l
        const int cin = kCin[l], cout = kCout[l];
        const int pairs = 9 * cin;
        cudaError_t de;
        if (LBM_DW_TC) {
            if (l == 0) de = launch_dw<2, 4>(N, N->x[0], g, B, cin, cout);
            else if (l == kLayers - 1) de = launch_dw<4, 2>(N, N->x[l], g, B, cin, cout);
            else de = launch_dw<4, 4>(N, N->x[l], g, B, cin, cout);
        } else {
            if (l == 0)
                dw_partial_kernel<2, 4><<<N->dw_blocks, 288, 0, N->stream>>>(
                    N->x[0], g, B, N->H, N->W, cin, cout, N->dw_partial, N->db_partial);
            else if (l == kLayers - 1)
                dw_partial_kernel<4, 2><<<N->dw_blocks, 288, 0, N->stream>>>(
                    N->x[l], g, B, N->H, N->W, cin, cout, N->dw_partial, N->db_partial);
            else
                dw_partial_kernel<4, 4><<<N->dw_blocks, 288, 0, N->stream>>>(
                    N->x[l], g, B, N->H, N->W, cin, cout, N->dw_partial, N->db_partial);
            de = cudaGetLastError();
        }
        if (de != cudaSuccess) { (void)cudaGetLastError(); return cfail(LBM_ERR_CUDA, cudaGetErrorString(de)); }
        reduce_partials_kernel<<<grid_of(pairs * cout, 256), 256, 0, N->stream>>>(
            N->dw_partial, N->dw_blocks, pairs * cout, N->grads + N->off_w[l]);
        CNN_CUDA(cudaGetLastError());
        reduce_partials_kernel<<<1, 64, 0, N->stream>>>(N->db_partial, N->dw_blocks, cout,
                                                        N->grads + N->off_b[l]);
        CNN_CUDA(cudaGetLastError());
        if (l == 0) break;
        // gradient wrt the layer's input, through GELU' of the previous layer
        ConvArgs a{};
        a.in = g;
        a.wpack = N->wd[l];
        a.x_out = N->gbuf[l];
        a.zprev = N->z[l - 1];
        a.B = B;
        a.H = N->H;
        a.W = N->W;
        a.err = N->err;
        cudaError_t e = (l == kLayers - 1) ? launch_conv<2, 32, 2>(N, a) : launch_conv<4, 32, 2>(N, a);
        if (e != cudaSuccess) { (void)cudaGetLastError(); return cfail(LBM_ERR_CUDA, cudaGetErrorString(e)); }
    }
    return LBM_OK;
}

int check_err(lbm_cnn* N) {
    int h = 0;
    CNN_CUDA(cudaMemcpyAsync(&h, N->err, sizeof(int), cudaMemcpyDeviceToHost, N->stream));
    CNN_CUDA(cudaStreamSynchronize(N->stream));
    if (h) {
        CNN_CUDA(cudaMemsetAsync(N->err, 0, sizeof(int), N->stream));
        return cfail(LBM_ERR_TIMEOUT, "a tensor-core wait timed out; results discarded");
    }
    return LBM_OK;
}

}  // namespace

extern "C" {

int lbm_cnn_create(int h, int w, int max_batch, uint64_t seed, lbm_cnn** out) {
    if (!out) return cfail(LBM_ERR_INVALID_ARGUMENT, "out must not be null");
    *out = nullptr;
    if (h < 1 || w < 1 || w % kTileM != 0 || max_batch < 1 || h > 65535 || max_batch > 65535)
        return cfail(LBM_ERR_INVALID_ARGUMENT, "need h >= 1, w a multiple of 128, max_batch >= 1");
    lbm_cnn* N = new lbm_cnn();
    N->H = h;
    N->W = w;
    N->maxB = max_batch;
    auto cleanup = [&](int rc) { lbm_cnn_destroy(N); return rc; };
    if (cudaGetDevice(&N->dev) != cudaSuccess) return cleanup(cfail(LBM_ERR_CUDA, "no device"));
    int n = 0;
    for (int l = 0; l < kLayers; ++l) {
        N->off_w[l] = n;
        n += 9 * kCin[l] * kCout[l];
        N->off_b[l] = n;
        n += kCout[l];
    }
    N->nparams = n;
    // He-style initial weights from a splitmix64 stream (host), zero biases.
    std::vector<float> p(n, 0.f);
    uint64_t state = seed;
    auto next = [&]() {
        uint64_t z = (state += 0x9E3779B97F4A7C15ull);
        z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
        z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
        z ^= z >> 31;
        return double(z >> 11) * (1.0 / 9007199254740992.0);
    };
    for (int l = 0; l < kLayers; ++l) {
        const double lim = std::sqrt(6.0 / (9.0 * kCin[l])) * (l == kLayers - 1 ? 0.1 : 1.0);
        for (int k = 0; k < 9 * kCin[l] * kCout[l]; ++k) p[N->off_w[l] + k] = float((2.0 * next() - 1.0) * lim);
    }
    cudaError_t e = cudaStreamCreateWithFlags(&N->own, cudaStreamNonBlocking);
    if (e != cudaSuccess) return cleanup(cfail(LBM_ERR_CUDA, cudaGetErrorString(e)));
    N->stream = N->own;
    auto alloc = [&](void** ptr, size_t bytes) -> int {
        cudaError_t r = cudaMalloc(ptr, bytes);
        if (r != cudaSuccess) {
            (void)cudaGetLastError();
            return cfail(r == cudaErrorMemoryAllocation ? LBM_ERR_OUT_OF_MEMORY : LBM_ERR_CUDA,
                         cudaGetErrorString(r));
        }
        return cudaMemsetAsync(*ptr, 0, bytes, N->stream) == cudaSuccess ? LBM_OK
                                                                         : cfail(LBM_ERR_CUDA, "memset");
    };
    int rc = 0;
    if ((rc = alloc((void**)&N->params, n * 4)) || (rc = alloc((void**)&N->grads, n * 4)) ||
        (rc = alloc((void**)&N->adam_m, n * 4)) || (rc = alloc((void**)&N->adam_v, n * 4)) ||
        (rc = alloc((void**)&N->err, 16)))
        return cleanup(rc);
    for (int l = 0; l < kLayers; ++l) {
        const size_t bf = size_t(9) * pad16(kCin[l]) * pad16(kCout[l]) * 2;
        if ((rc = alloc((void**)&N->wf[l], bf))) return cleanup(rc);
        if (l > 0 && (rc = alloc((void**)&N->wd[l], size_t(9) * pad16(kCout[l]) * pad16(kCin[l]) * 2)))
            return cleanup(rc);
        if ((rc = alloc((void**)&N->x[l], cb8_bytes(N, max_batch, cbi_of(kCin[l]))))) return cleanup(rc);
        if (l < kLayers - 1 && (rc = alloc((void**)&N->z[l], cb8_bytes(N, max_batch, cbi_of(kCout[l])))))
            return cleanup(rc);
        if (l > 0 && (rc = alloc((void**)&N->gbuf[l], cb8_bytes(N, max_batch, cbi_of(kCin[l])))))
            return cleanup(rc);
    }
    if ((rc = alloc((void**)&N->gbuf[kLayers], cb8_bytes(N, max_batch, 2)))) return cleanup(rc);
    if ((rc = alloc((void**)&N->out, size_t(max_batch) * 9 * h * w * 4))) return cleanup(rc);
    int sms = 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, N->dev);
    N->dw_blocks = std::max(1, sms * 2);
    if ((rc = alloc((void**)&N->dw_partial, size_t(N->dw_blocks) * 9 * 32 * 32 * 4))) return cleanup(rc);
    if ((rc = alloc((void**)&N->db_partial, size_t(N->dw_blocks) * 32 * 4))) return cleanup(rc);
    if ((rc = alloc((void**)&N->loss_partial, 1024 * 8))) return cleanup(rc);
    e = cudaMemcpyAsync(N->params, p.data(), n * 4, cudaMemcpyHostToDevice, N->stream);
    if (e != cudaSuccess) return cleanup(cfail(LBM_ERR_CUDA, cudaGetErrorString(e)));
    if ((rc = repack(N))) return cleanup(rc);
    e = cudaStreamSynchronize(N->stream);
    if (e != cudaSuccess) return cleanup(cfail(LBM_ERR_CUDA, cudaGetErrorString(e)));
    *out = N;
    return LBM_OK;
}

int lbm_cnn_destroy(lbm_cnn* N) {
    if (!N) return LBM_OK;
    if (N->stream) cudaStreamSynchronize(N->stream);
    void* ptrs[] = {N->params, N->grads, N->adam_m, N->adam_v, N->err, N->out, N->dw_partial,
                    N->db_partial, N->loss_partial, N->feat};
    for (void* q : ptrs)
        if (q) cudaFree(q);
    for (int l = 0; l < kLayers; ++l) {
        if (N->wf[l]) cudaFree(N->wf[l]);
        if (N->wd[l]) cudaFree(N->wd[l]);
        if (N->x[l]) cudaFree(N->x[l]);
        if (N->z[l]) cudaFree(N->z[l]);
    }
    for (auto* g : N->gbuf)
        if (g) cudaFree(g);
    if (N->own) cudaStreamDestroy(N->own);
    delete N;
    return LBM_OK;
}

int lbm_cnn_param_count(lbm_cnn* N, int64_t* n) {
    if (!N || !n) return cfail(LBM_ERR_INVALID_ARGUMENT, "null argument");
    *n = N->nparams;
    return LBM_OK;
}

int lbm_cnn_get_params(lbm_cnn* N, float* host) {
    if (!N || !host) return cfail(LBM_ERR_INVALID_ARGUMENT, "null argument");
    CNN_CUDA(cudaMemcpyAsync(host, N->params, size_t(N->nparams) * 4, cudaMemcpyDeviceToHost, N->stream));
    CNN_CUDA(cudaStreamSynchronize(N->stream));
    return LBM_OK;
}

int lbm_cnn_set_params(lbm_cnn* N, const float* host) {
    if (!N || !host) return cfail(LBM_ERR_INVALID_ARGUMENT, "null argument");
    CNN_CUDA(cudaMemcpyAsync(N->params, host, size_t(N->nparams) * 4, cudaMemcpyHostToDevice, N->stream));
    if (int rc = repack(N)) return rc;
    CNN_CUDA(cudaStreamSynchronize(N->stream));
    return LBM_OK;
}

int lbm_cnn_forward(lbm_cnn* N, const float* in_dev, int batch, float* out_dev) {
    if (!N || !in_dev || !out_dev) return cfail(LBM_ERR_INVALID_ARGUMENT, "null argument");
    if (batch < 1 || batch > N->maxB) return cfail(LBM_ERR_INVALID_ARGUMENT, "batch out of range");
    nchw_to_cb8_kernel<<<grid_of(int64_t(batch) * N->H * N->W * 2, 256), 256, 0, N->stream>>>(
        in_dev, batch, 4, N->H, N->W, 2, N->x[0]);
    CNN_CUDA(cudaGetLastError());
    if (int rc = forward_impl(N, batch, false)) return rc;
    CNN_CUDA(cudaMemcpyAsync(out_dev, N->out, size_t(batch) * 9 * N->H * N->W * 4,
                             cudaMemcpyDeviceToDevice, N->stream));
    return check_err(N);
}

int lbm_cnn_gradients(lbm_cnn* N, const float* in_dev, const float* target_dev, int batch,
                      float* loss, float* grads_host) {
    if (!N || !in_dev || !target_dev) return cfail(LBM_ERR_INVALID_ARGUMENT, "null argument");
    if (batch < 1 || batch > N->maxB) return cfail(LBM_ERR_INVALID_ARGUMENT, "batch out of range");
    nchw_to_cb8_kernel<<<grid_of(int64_t(batch) * N->H * N->W * 2, 256), 256, 0, N->stream>>>(
        in_dev, batch, 4, N->H, N->W, 2, N->x[0]);
    CNN_CUDA(cudaGetLastError());
    if (int rc = forward_impl(N, batch, true)) return rc;
    const double count = double(batch) * 9 * N->H * N->W;
    mse_kernel<<<1024, 256, 0, N->stream>>>(N->out, target_dev, batch, 9, N->H, N->W,
                                            float(2.0 / count), N->gbuf[kLayers], N->loss_partial);
    CNN_CUDA(cudaGetLastError());
    if (int rc = backward_impl(N, batch)) return rc;
    if (loss) {
        std::vector<double> part(1024);
        CNN_CUDA(cudaMemcpyAsync(part.data(), N->loss_partial, 1024 * 8, cudaMemcpyDeviceToHost, N->stream));
        CNN_CUDA(cudaStreamSynchronize(N->stream));
        double s = 0.0;
        for (double v : part) s += v;
        *loss = float(s / count);
    }
    if (grads_host)
        CNN_CUDA(cudaMemcpyAsync(grads_host, N->grads, size_t(N->nparams) * 4, cudaMemcpyDeviceToHost,
                                 N->stream));
    return check_err(N);
}

int lbm_cnn_train_step(lbm_cnn* N, const float* in_dev, const float* target_dev, int batch,
                       float lr, float* loss) {
    if (int rc = lbm_cnn_gradients(N, in_dev, target_dev, batch, loss, nullptr)) return rc;
    N->adam_t += 1;
    const float b1 = 0.9f, b2 = 0.999f;
    const float c1 = 1.f - std::pow(b1, float(N->adam_t)), c2 = 1.f - std::pow(b2, float(N->adam_t));
    adam_kernel<<<grid_of(N->nparams, 256), 256, 0, N->stream>>>(N->params, N->grads, N->adam_m,
                                                                  N->adam_v, N->nparams, lr, b1, b2,
                                                                  1e-8f, c1, c2);
    CNN_CUDA(cudaGetLastError());
    if (int rc = repack(N)) return rc;
    return LBM_OK;
}

int lbm_selftest_wait_timeout(uint32_t polls, int* timed_out) {
    if (!timed_out) return cfail(LBM_ERR_INVALID_ARGUMENT, "null argument");
    if (polls < 1 || polls > kWaitPolls) return cfail(LBM_ERR_INVALID_ARGUMENT, "polls out of range");
    *timed_out = 0;
    int* d = nullptr;
    CNN_CUDA(cudaMalloc(&d, sizeof(int)));
    cudaError_t e = cudaMemset(d, 0, sizeof(int));
    if (e == cudaSuccess) {
        wait_probe_kernel<<<1, 32>>>(d, polls);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaMemcpy(timed_out, d, sizeof(int), cudaMemcpyDeviceToHost);
    cudaFree(d);
    CNN_CUDA(e);
    return LBM_OK;
}

int lbm_cnn_save(lbm_cnn* N, const char* path) {
    if (!N || !path) return cfail(LBM_ERR_INVALID_ARGUMENT, "null argument");
    std::vector<float> p(N->nparams);
    if (int rc = lbm_cnn_get_params(N, p.data())) return rc;
    FILE* fp = std::fopen(path, "wb");
    if (!fp) return cfail(LBM_ERR_INVALID_ARGUMENT, std::string("cannot open ") + path);
    const int64_t n = N->nparams;
    const bool ok = std::fwrite(kCnnMagic, 1, 8, fp) == 8 && std::fwrite(&n, 8, 1, fp) == 1 &&
                    std::fwrite(p.data(), 4, p.size(), fp) == p.size();
    if (std::fclose(fp) != 0 || !ok) return cfail(LBM_ERR_INVALID_ARGUMENT, "write failed");
    return LBM_OK;
}

int lbm_cnn_load(lbm_cnn* N, const char* path) {
    if (!N || !path) return cfail(LBM_ERR_INVALID_ARGUMENT, "null argument");
    FILE* fp = std::fopen(path, "rb");
    if (!fp) return cfail(LBM_ERR_INVALID_ARGUMENT, std::string("cannot open ") + path);
    char magic[8] = {};
    int64_t n = 0;
    std::vector<float> p(N->nparams);
    const bool ok = std::fread(magic, 1, 8, fp) == 8 && std::memcmp(magic, kCnnMagic, 8) == 0 &&
                    std::fread(&n, 8, 1, fp) == 1 && n == N->nparams &&
                    std::fread(p.data(), 4, p.size(), fp) == p.size();
    std::fclose(fp);
    if (!ok) return cfail(LBM_ERR_INVALID_ARGUMENT, "not a weight file of this network");
    return lbm_cnn_set_params(N, p.data());
}

int lbm_coarse_run(lbm_lattice* lat, lbm_cnn* N, int nsteps, int k, float s_rho, float s_u,
                   float scale, float max_abs, int check_every, float mass_tolerance,
                   int64_t* fallback_step) {
    if (!lat || !N || !fallback_step) return cfail(LBM_ERR_INVALID_ARGUMENT, "null argument");
    *fallback_step = -1;
    if (nsteps < 0 || k < 1 || check_every < 0 || !(mass_tolerance > 0.f))
        return cfail(LBM_ERR_INVALID_ARGUMENT, "need nsteps >= 0, k >= 1, check_every >= 0, "
                                               "mass_tolerance > 0");
    if (lat->precision != LBM_F32 || lat->w != N->W || lat->h != N->H)
        return cfail(LBM_ERR_INVALID_ARGUMENT, "need an f32 lattice of the network's size");
    if (!N->feat) {
        CNN_CUDA(cudaMalloc(&N->feat, size_t(4) * N->H * N->W * 4));
        CNN_CUDA(cudaMemsetAsync(N->feat, 0, size_t(4) * N->H * N->W * 4, N->stream));
    }
    CNN_CUDA(cudaStreamSynchronize(N->stream));
    const cudaStream_t saved = N->stream;
    N->stream = lat->stream;                       // one stream orders step, net and apply
    auto finish = [&](int rc) {
        N->stream = saved;
        return rc;
    };
    lbm_health h0{};
    if (int rc = lbm_check(lat, &h0)) return finish(rc);
    int done = 0, corrections = 0;
    while (done < nsteps) {
        const int n = std::min(k, nsteps - done);
        if (int rc = lbm_step(lat, n)) return finish(rc);
        done += n;
        if (n < k) break;
        if (int rc = lbm_coarse_features(lat, s_rho, s_u, 0, N->feat)) return finish(rc);
        nchw_to_cb8_kernel<<<grid_of(int64_t(N->H) * N->W * 2, 256), 256, 0, N->stream>>>(
            N->feat, 1, 4, N->H, N->W, 2, N->x[0]);
        if (cudaGetLastError() != cudaSuccess) return finish(cfail(LBM_ERR_CUDA, "features launch"));
        if (int rc = forward_impl(N, 1, false)) return finish(rc);
        if (int rc = lbm_coarse_apply(lat, N->out, 0, scale, max_abs)) return finish(rc);
        ++corrections;
        if (check_every > 0 && corrections % check_every == 0) {
            // the periodic check: an unstable state or a mass drift past the
            // tolerance ends the coarse run; the caller continues on the fine grid
            lbm_health h{};
            if (int rc = lbm_check(lat, &h)) return finish(rc);
            if (h.unstable || std::fabs(h.mass - h0.mass) > double(mass_tolerance) * std::fabs(h0.mass)) {
                *fallback_step = lat->steps;
                break;
            }
        }
    }
    return finish(check_err(N));
}

int lbm_cnn_set_stream(lbm_cnn* N, void* stream) {
    if (!N) return cfail(LBM_ERR_INVALID_ARGUMENT, "null argument");
    CNN_CUDA(cudaStreamSynchronize(N->stream));
    N->stream = stream ? static_cast<cudaStream_t>(stream) : N->own;
    return LBM_OK;
}

int lbm_cnn_synchronize(lbm_cnn* N) {
    if (!N) return cfail(LBM_ERR_INVALID_ARGUMENT, "null argument");
    CNN_CUDA(cudaStreamSynchronize(N->stream));
    return LBM_OK;
}

}  // extern "C"
