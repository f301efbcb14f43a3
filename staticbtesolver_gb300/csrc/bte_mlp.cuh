// bte_mlp.cuh -- the per-cell MLP of the learned outer-iteration accelerator.
//
// Network: 8 inputs -> 128 -> 128 -> 128 -> 1, ReLU, BF16 weights and
// activations, FP32 accumulation on the tensor cores (mma.sync m16n8k16,
// one warp per 16 samples).  Parameters are kept as FP32 "master" values in
// one flat array (layout below) and packed to BF16 for the kernels.
//
// Flat FP32 parameter layout (row-major [in][out] weights):
//   W1[8][128] b1[128] W2[128][128] b2[128] W3[128][128] b3[128] W4[128][1] b4[1]
#pragma once
#include <cuda_bf16.h>
#include <stdint.h>

namespace bte {
namespace mlp {

constexpr int IN = 8, H = 128, IN_PAD = 16;
constexpr int OFF_W1 = 0, OFF_B1 = OFF_W1 + IN * H, OFF_W2 = OFF_B1 + H, OFF_B2 = OFF_W2 + H * H;
constexpr int OFF_W3 = OFF_B2 + H, OFF_B3 = OFF_W3 + H * H, OFF_W4 = OFF_B3 + H, OFF_B4 = OFF_W4 + H;
constexpr int NPARAM = OFF_B4 + 1;  // 34305

// BF16 weights in the layouts the kernels read, all "out-major" ([out][in]):
// w1t[128][16] (inputs 8..15 zero), w2t[128][128], w3t[128][128], w4t[8][128]
// (outputs 1..7 zero), and FP32 biases.
constexpr int PK_W1 = 0, PK_W2 = PK_W1 + H * IN_PAD, PK_W3 = PK_W2 + H * H, PK_W4 = PK_W3 + H * H;
constexpr int PK_N = PK_W4 + 8 * H;  // bf16 elements

__device__ __forceinline__ uint32_t pack2(float lo, float hi) {
    __nv_bfloat162 v = __floats2bfloat162_rn(lo, hi);
    return *reinterpret_cast<uint32_t*>(&v);
}
__device__ __forceinline__ uint32_t pack2(__nv_bfloat16 lo, __nv_bfloat16 hi) {
    __nv_bfloat162 v;
    v.x = lo;
    v.y = hi;
    return *reinterpret_cast<uint32_t*>(&v);
}

// D = A(16x16, row) * B(16x8, col) + D, BF16 inputs, FP32 accumulate.
__device__ __forceinline__ void mma16816(float (&c)[4], const uint32_t (&a)[4], uint32_t b0, uint32_t b1) {
    asm volatile(
        "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
        "{%0,%1,%2,%3};\n"
        : "+f"(c[0]), "+f"(c[1]), "+f"(c[2]), "+f"(c[3])
        : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}

// FP32 master parameters -> BF16 out-major weights.
__global__ void k_pack(const float* __restrict__ p, __nv_bfloat16* __restrict__ w) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < H * IN_PAD) {  // w1t[o][k]
        const int o = i / IN_PAD, k = i % IN_PAD;
        w[PK_W1 + i] = __float2bfloat16(k < IN ? p[OFF_W1 + k * H + o] : 0.0f);
    }
    if (i < H * H) {
        const int o = i / H, k = i % H;
        w[PK_W2 + i] = __float2bfloat16(p[OFF_W2 + k * H + o]);
        w[PK_W3 + i] = __float2bfloat16(p[OFF_W3 + k * H + o]);
    }
    if (i < 8 * H) {
        const int o = i / H, k = i % H;
        w[PK_W4 + i] = __float2bfloat16(o == 0 ? p[OFF_W4 + k] : 0.0f);
    }
}

// Shared-memory image of the packed weights and the biases.
struct Smem {
    __nv_bfloat16 w[PK_N];
    float b[3 * H + 1];
};

__device__ __forceinline__ void load_smem(Smem& s, const __nv_bfloat16* __restrict__ w, const float* __restrict__ p) {
    const uint32_t* src = reinterpret_cast<const uint32_t*>(w);
    uint32_t* dst = reinterpret_cast<uint32_t*>(s.w);
    for (int i = threadIdx.x; i < PK_N / 2; i += blockDim.x) dst[i] = src[i];
    for (int i = threadIdx.x; i < H; i += blockDim.x) {
        s.b[i] = p[OFF_B1 + i];
        s.b[H + i] = p[OFF_B2 + i];
        s.b[2 * H + i] = p[OFF_B3 + i];
    }
    if (threadIdx.x == 0) s.b[3 * H] = p[OFF_B4];
    __syncthreads();
}

// One hidden layer for this warp's 16 rows: acc = A(16 x K) * W^T, K = 16*kt.
// wt is [128][ldk] out-major; a[kk] are the A fragments of k-tile kk.
template <int KT>
__device__ __forceinline__ void layer(float (&acc)[16][4], const uint32_t (&a)[KT][4], const __nv_bfloat16* wt, int ldk,
                                      int g, int t) {
#pragma unroll
    for (int j = 0; j < 16; ++j) {
        acc[j][0] = acc[j][1] = acc[j][2] = acc[j][3] = 0.0f;
        const __nv_bfloat16* row = wt + (size_t)(8 * j + g) * ldk + 2 * t;
#pragma unroll
        for (int kk = 0; kk < KT; ++kk) {
            const uint32_t b0 = *reinterpret_cast<const uint32_t*>(row + 16 * kk);
            const uint32_t b1 = *reinterpret_cast<const uint32_t*>(row + 16 * kk + 8);
            mma16816(acc[j], a[kk], b0, b1);
        }
    }
}

// bias + ReLU, then repack as the next layer's A fragments (two adjacent
// n-tiles of the accumulator are exactly one 16-wide k-tile of A).
__device__ __forceinline__ void relu_pack(float (&acc)[16][4], const float* bias, int t, uint32_t (&h)[8][4]) {
#pragma unroll
    for (int j = 0; j < 16; ++j) {
        const float b0 = bias[8 * j + 2 * t], b1 = bias[8 * j + 2 * t + 1];
        acc[j][0] = fmaxf(acc[j][0] + b0, 0.0f);
        acc[j][1] = fmaxf(acc[j][1] + b1, 0.0f);
        acc[j][2] = fmaxf(acc[j][2] + b0, 0.0f);
        acc[j][3] = fmaxf(acc[j][3] + b1, 0.0f);
    }
#pragma unroll
    for (int kk = 0; kk < 8; ++kk) {
        h[kk][0] = pack2(acc[2 * kk][0], acc[2 * kk][1]);
        h[kk][1] = pack2(acc[2 * kk][2], acc[2 * kk][3]);
        h[kk][2] = pack2(acc[2 * kk + 1][0], acc[2 * kk + 1][1]);
        h[kk][3] = pack2(acc[2 * kk + 1][2], acc[2 * kk + 1][3]);
    }
}

// Store A fragments of a 16 x 128 activation tile to act[M][128] (bf16).
__device__ __forceinline__ void store_frag(const uint32_t (&h)[8][4], __nv_bfloat16* act, int r0, int g, int t, int M) {
#pragma unroll
    for (int kk = 0; kk < 8; ++kk) {
        const int c0 = 16 * kk + 2 * t;
        if (r0 + g < M) {
            *reinterpret_cast<uint32_t*>(act + (size_t)(r0 + g) * H + c0) = h[kk][0];
            *reinterpret_cast<uint32_t*>(act + (size_t)(r0 + g) * H + c0 + 8) = h[kk][2];
        }
        if (r0 + g + 8 < M) {
            *reinterpret_cast<uint32_t*>(act + (size_t)(r0 + g + 8) * H + c0) = h[kk][1];
            *reinterpret_cast<uint32_t*>(act + (size_t)(r0 + g + 8) * H + c0 + 8) = h[kk][3];
        }
    }
}

// Forward: x[M][16] bf16 (features 8..15 zero) -> y[M] fp32.  If act != null
// the post-ReLU activations of the three hidden layers are stored to
// act[3][M][128] for the backward pass.  Rows beyond M read as zero.
__global__ void __launch_bounds__(128) k_forward(const __nv_bfloat16* __restrict__ x, int M,
                                                 const __nv_bfloat16* __restrict__ w, const float* __restrict__ p,
                                                 float* __restrict__ y, __nv_bfloat16* __restrict__ act) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    Smem& s = *reinterpret_cast<Smem*>(smem_raw);
    load_smem(s, w, p);
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int g = lane >> 2, t = lane & 3;
    const int nwarps = gridDim.x * (blockDim.x >> 5);
    for (int r0 = (blockIdx.x * (blockDim.x >> 5) + warp) * 16; r0 < M; r0 += nwarps * 16) {
        uint32_t a1[1][4];
        {
            const uint32_t* xr = reinterpret_cast<const uint32_t*>(x);
            const int ra = r0 + g, rb = r0 + g + 8;
            a1[0][0] = ra < M ? xr[(size_t)ra * 8 + t] : 0u;
            a1[0][1] = rb < M ? xr[(size_t)rb * 8 + t] : 0u;
            a1[0][2] = ra < M ? xr[(size_t)ra * 8 + 4 + t] : 0u;
            a1[0][3] = rb < M ? xr[(size_t)rb * 8 + 4 + t] : 0u;
        }
        float acc[16][4];
        uint32_t h[8][4];
        layer<1>(acc, a1, s.w + PK_W1, IN_PAD, g, t);
        relu_pack(acc, s.b, t, h);
        if (act) store_frag(h, act, r0, g, t, M);
        layer<8>(acc, h, s.w + PK_W2, H, g, t);
        relu_pack(acc, s.b + H, t, h);
        if (act) store_frag(h, act + (size_t)M * H, r0, g, t, M);
        layer<8>(acc, h, s.w + PK_W3, H, g, t);
        relu_pack(acc, s.b + 2 * H, t, h);
        if (act) store_frag(h, act + (size_t)2 * M * H, r0, g, t, M);
        float o[4] = {0, 0, 0, 0};
        const __nv_bfloat16* row = s.w + PK_W4 + (size_t)g * H + 2 * t;
#pragma unroll
        for (int kk = 0; kk < 8; ++kk) {
            const uint32_t b0 = *reinterpret_cast<const uint32_t*>(row + 16 * kk);
            const uint32_t b1 = *reinterpret_cast<const uint32_t*>(row + 16 * kk + 8);
            mma16816(o, h[kk], b0, b1);
        }
        if (t == 0) {  // column 0 of the 16 x 8 output tile
            if (r0 + g < M) y[r0 + g] = o[0] + s.b[3 * H];
            if (r0 + g + 8 < M) y[r0 + g + 8] = o[2] + s.b[3 * H];
        }
    }
}

// Loss L = mean over rows of 0.5 (y - target)^2 (targets clipped by the
// caller); dy = (y - target) / M; per-block partial sums of the loss.
__global__ void k_loss(const float* __restrict__ y, const float* __restrict__ target, int M, float* __restrict__ dy,
                       double* __restrict__ part) {
    __shared__ double sm[8];
    double acc = 0.0;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < M; i += gridDim.x * blockDim.x) {
        const float d = y[i] - target[i];
        dy[i] = d / (float)M;
        acc += 0.5 * (double)d * d;
    }
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, o);
    if ((threadIdx.x & 31) == 0) sm[threadIdx.x >> 5] = acc;
    __syncthreads();
    if (threadIdx.x == 0) {
        double s = 0;
        for (int w = 0; w < (int)(blockDim.x >> 5); ++w) s += sm[w];
        part[blockIdx.x] = s / M;
    }
}

// Backward through the hidden layers (activations from the forward pass):
//   dh3 = dy W4^T . [h3 > 0];  dh2 = dh3 W3^T . [h2 > 0];  dh1 = dh2 W2^T . [h1 > 0]
// The W^T products read the weights in [in][out] order (wi2, wi3, both
// [128][128] bf16) so each B fragment pair is contiguous.  Outputs dh[3][M][128] bf16.
__global__ void __launch_bounds__(128) k_backward_data(const float* __restrict__ dy, int M,
                                                       const __nv_bfloat16* __restrict__ act,
                                                       const __nv_bfloat16* __restrict__ wi,  // [2][128][128]: W2, W3 as [in][out]
                                                       const float* __restrict__ p, __nv_bfloat16* __restrict__ dh) {
    extern __shared__ __align__(16) unsigned char smem_bwd[];  // BWD_SMEM bytes
    __nv_bfloat16* sw = reinterpret_cast<__nv_bfloat16*>(smem_bwd);
    float* w4 = reinterpret_cast<float*>(smem_bwd + sizeof(__nv_bfloat16) * 2 * H * H);
    {
        const uint32_t* src = reinterpret_cast<const uint32_t*>(wi);
        uint32_t* dst = reinterpret_cast<uint32_t*>(sw);
        for (int i = threadIdx.x; i < H * H; i += blockDim.x) dst[i] = src[i];
        for (int i = threadIdx.x; i < H; i += blockDim.x) w4[i] = p[OFF_W4 + i];
        __syncthreads();
    }
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int g = lane >> 2, t = lane & 3;
    const int nwarps = gridDim.x * (blockDim.x >> 5);
    for (int r0 = (blockIdx.x * (blockDim.x >> 5) + warp) * 16; r0 < M; r0 += nwarps * 16) {
        const int ra = r0 + g, rb = r0 + g + 8;
        const float dya = ra < M ? dy[ra] : 0.0f, dyb = rb < M ? dy[rb] : 0.0f;
        auto act_at = [&](int layer_i, int r, int c) -> float {
            return r < M ? __bfloat162float(act[((size_t)layer_i * M + r) * H + c]) : 0.0f;
        };
        // dh3 in A-fragment form directly
        uint32_t d[8][4];
#pragma unroll
        for (int kk = 0; kk < 8; ++kk) {
            const int c0 = 16 * kk + 2 * t, c1 = c0 + 8;
            float v[8];
            v[0] = act_at(2, ra, c0) > 0.f ? dya * w4[c0] : 0.f;
            v[1] = act_at(2, ra, c0 + 1) > 0.f ? dya * w4[c0 + 1] : 0.f;
            v[2] = act_at(2, rb, c0) > 0.f ? dyb * w4[c0] : 0.f;
            v[3] = act_at(2, rb, c0 + 1) > 0.f ? dyb * w4[c0 + 1] : 0.f;
            v[4] = act_at(2, ra, c1) > 0.f ? dya * w4[c1] : 0.f;
            v[5] = act_at(2, ra, c1 + 1) > 0.f ? dya * w4[c1 + 1] : 0.f;
            v[6] = act_at(2, rb, c1) > 0.f ? dyb * w4[c1] : 0.f;
            v[7] = act_at(2, rb, c1 + 1) > 0.f ? dyb * w4[c1 + 1] : 0.f;
            d[kk][0] = pack2(v[0], v[1]);
            d[kk][1] = pack2(v[2], v[3]);
            d[kk][2] = pack2(v[4], v[5]);
            d[kk][3] = pack2(v[6], v[7]);
        }
        store_frag(d, dh + (size_t)2 * M * H, r0, g, t, M);
        // dh2 = dh3 W3^T, then dh1 = dh2 W2^T; masks from h2, h1
        for (int li = 1; li >= 0; --li) {
            float acc[16][4];
            layer<8>(acc, d, sw + (size_t)li * H * H, H, g, t);  // B[k=out][n=in] = W[in][out]: rows of wi are "in"
#pragma unroll
            for (int j = 0; j < 16; ++j) {
                const int c = 8 * j + 2 * t;
                if (act_at(li, ra, c) <= 0.f) acc[j][0] = 0.f;
                if (act_at(li, ra, c + 1) <= 0.f) acc[j][1] = 0.f;
                if (act_at(li, rb, c) <= 0.f) acc[j][2] = 0.f;
                if (act_at(li, rb, c + 1) <= 0.f) acc[j][3] = 0.f;
            }
#pragma unroll
            for (int kk = 0; kk < 8; ++kk) {
                d[kk][0] = pack2(acc[2 * kk][0], acc[2 * kk][1]);
                d[kk][1] = pack2(acc[2 * kk][2], acc[2 * kk][3]);
                d[kk][2] = pack2(acc[2 * kk + 1][0], acc[2 * kk + 1][1]);
                d[kk][3] = pack2(acc[2 * kk + 1][2], acc[2 * kk + 1][3]);
            }
            store_frag(d, dh + (size_t)li * M * H, r0, g, t, M);
        }
    }
}

constexpr size_t FWD_SMEM = sizeof(Smem);
constexpr size_t BWD_SMEM = sizeof(__nv_bfloat16) * 2 * H * H + sizeof(float) * H;

// FP32 master weights -> BF16 [in][out] copies of W2 and W3 for k_backward_data.
__global__ void k_pack_in_major(const float* __restrict__ p, __nv_bfloat16* __restrict__ wi) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= H * H) return;
    wi[i] = __float2bfloat16(p[OFF_W2 + i]);
    wi[H * H + i] = __float2bfloat16(p[OFF_W3 + i]);
}

// Weight gradients for one layer over a slice of rows:
//   part[slice][in][out] = sum_{rows of slice} a[r][in] * d[r][out]
// a: [M][lda] bf16 (lda = 16 for the input layer, 128 otherwise), d: [M][128]
// bf16.  Block = 8 warps; warp w owns in-rows 16*(w % (KIN/16)) .. and out
// columns 64*(w / (KIN/16)) ...  The transposed A operand is staged through
// shared memory.  Rows are taken in slices of 64.
template <int KIN>
__global__ void __launch_bounds__(256) k_weight_grad(const __nv_bfloat16* __restrict__ a, int lda,
                                                     const __nv_bfloat16* __restrict__ d, int M, int rows_per_slice,
                                                     float* __restrict__ part) {
    __shared__ __align__(16) __nv_bfloat16 sa[64][KIN + 8];
    __shared__ __align__(16) __nv_bfloat16 sd[64][H + 8];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int g = lane >> 2, t = lane & 3;
    constexpr int MT = KIN / 16;          // 16-row tiles of "in"
    constexpr int NW_OUT = 8 / MT;        // warps sharing one in-tile
    const int mt = warp % MT;
    constexpr int n_span = H / NW_OUT;    // out columns per warp
    const int n0 = (warp / MT) * n_span;
    float acc[16][4];
#pragma unroll
    for (int j = 0; j < 16; ++j) acc[j][0] = acc[j][1] = acc[j][2] = acc[j][3] = 0.f;
    const int r_begin = blockIdx.x * rows_per_slice;
    const int r_end = min(M, r_begin + rows_per_slice);
    for (int rb = r_begin; rb < r_end; rb += 64) {
        __syncthreads();
        for (int i = threadIdx.x; i < 64 * KIN; i += blockDim.x) {
            const int r = i / KIN, c = i % KIN;
            sa[r][c] = (rb + r < r_end) ? a[(size_t)(rb + r) * lda + c] : __float2bfloat16(0.f);
        }
        for (int i = threadIdx.x; i < 64 * H; i += blockDim.x) {
            const int r = i / H, c = i % H;
            sd[r][c] = (rb + r < r_end) ? d[(size_t)(rb + r) * H + c] : __float2bfloat16(0.f);
        }
        __syncthreads();
#pragma unroll
        for (int ks = 0; ks < 4; ++ks) {  // 16 rows per k-step
            const int k0 = 16 * ks;
            uint32_t af[4];
            const int m = 16 * mt + g;
            af[0] = pack2(sa[k0 + 2 * t][m], sa[k0 + 2 * t + 1][m]);
            af[1] = pack2(sa[k0 + 2 * t][m + 8], sa[k0 + 2 * t + 1][m + 8]);
            af[2] = pack2(sa[k0 + 2 * t + 8][m], sa[k0 + 2 * t + 9][m]);
            af[3] = pack2(sa[k0 + 2 * t + 8][m + 8], sa[k0 + 2 * t + 9][m + 8]);
#pragma unroll
            for (int j = 0; j < n_span / 8; ++j) {
                const int n = n0 + 8 * j + g;
                const uint32_t b0 = pack2(sd[k0 + 2 * t][n], sd[k0 + 2 * t + 1][n]);
                const uint32_t b1 = pack2(sd[k0 + 2 * t + 8][n], sd[k0 + 2 * t + 9][n]);
                mma16816(acc[j], af, b0, b1);
            }
        }
    }
    float* out = part + (size_t)blockIdx.x * KIN * H;
#pragma unroll
    for (int j = 0; j < n_span / 8; ++j) {
        const int c = n0 + 8 * j + 2 * t;
        const int r = 16 * mt + g;
        out[(size_t)r * H + c] = acc[j][0];
        out[(size_t)r * H + c + 1] = acc[j][1];
        out[(size_t)(r + 8) * H + c] = acc[j][2];
        out[(size_t)(r + 8) * H + c + 1] = acc[j][3];
    }
}

// Gradient assembly into the flat FP32 layout:
//   weights: sum over slices of part (fixed order); W4[k] = sum_r h3[r][k] dy[r];
//   biases: b_l[o] = sum_r dh_l[r][o]; b4 = sum_r dy[r].
// One thread per parameter.
__global__ void k_grad_assemble(const float* __restrict__ p1, const float* __restrict__ p2,
                                const float* __restrict__ p3, int nslices, const __nv_bfloat16* __restrict__ act,
                                const __nv_bfloat16* __restrict__ dh, const float* __restrict__ dy, int M,
                                float* __restrict__ grad) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= NPARAM) return;
    double s = 0.0;
    if (i < OFF_B1) {  // W1[k][o], part1 is [slice][16][128]
        const int k = i / H, o = i % H;
        for (int q = 0; q < nslices; ++q) s += p1[((size_t)q * IN_PAD + k) * H + o];
    } else if (i < OFF_W2) {
        const int o = i - OFF_B1;
        for (int r = 0; r < M; ++r) s += __bfloat162float(dh[(size_t)r * H + o]);
    } else if (i < OFF_B2) {
        const int k = (i - OFF_W2) / H, o = (i - OFF_W2) % H;
        for (int q = 0; q < nslices; ++q) s += p2[((size_t)q * H + k) * H + o];
    } else if (i < OFF_W3) {
        const int o = i - OFF_B2;
        for (int r = 0; r < M; ++r) s += __bfloat162float(dh[((size_t)M + r) * H + o]);
    } else if (i < OFF_B3) {
        const int k = (i - OFF_W3) / H, o = (i - OFF_W3) % H;
        for (int q = 0; q < nslices; ++q) s += p3[((size_t)q * H + k) * H + o];
    } else if (i < OFF_W4) {
        const int o = i - OFF_B3;
        for (int r = 0; r < M; ++r) s += __bfloat162float(dh[((size_t)2 * M + r) * H + o]);
    } else if (i < OFF_B4) {
        const int k = i - OFF_W4;
        for (int r = 0; r < M; ++r) s += (double)__bfloat162float(act[((size_t)2 * M + r) * H + k]) * dy[r];
    } else {
        for (int r = 0; r < M; ++r) s += dy[r];
    }
    grad[i] = (float)s;
}

// Adam (Kingma & Ba) on the FP32 master parameters.
__global__ void k_adam(float* __restrict__ p, const float* __restrict__ grad, float* __restrict__ m,
                       float* __restrict__ v, float lr, float b1, float b2, float eps, float c1, float c2) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= NPARAM) return;
    const float gr = grad[i];
    const float mi = b1 * m[i] + (1.f - b1) * gr;
    const float vi = b2 * v[i] + (1.f - b2) * gr * gr;
    m[i] = mi;
    v[i] = vi;
    p[i] -= lr * (mi / c1) / (sqrtf(vi / c2) + eps);
}

}  // namespace mlp
}  // namespace bte

namespace bte {
namespace mlp {

// FP32 features [M][8] -> BF16 MLP input rows [M][16] (columns 8..15 zero).
__global__ void k_features_bf16(const float* __restrict__ X, int M, __nv_bfloat16* __restrict__ x) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= M * IN_PAD) return;
    const int r = i / IN_PAD, c = i % IN_PAD;
    x[i] = __float2bfloat16(c < IN ? X[(size_t)r * IN + c] : 0.0f);
}

// Gather a minibatch: rows idx[0..B) of x / Y.
__global__ void k_gather(const __nv_bfloat16* __restrict__ x, const float* __restrict__ Y, const int* __restrict__ idx,
                         int B, __nv_bfloat16* __restrict__ xb, float* __restrict__ yb) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= B * IN_PAD) return;
    const int r = i / IN_PAD, c = i % IN_PAD;
    xb[i] = x[(size_t)idx[r] * IN_PAD + c];
    if (c == 0) yb[r] = Y[idx[r]];
}

// Geometry constants of the accelerator's features.
struct FeatureGeom {
    const double* centroid;  // [n][3]
    const double* volume;    // [n]
    double vmean, xmin, xspan, ymin, yspan, kn_num, inv_dim, T_ref, dT_bc;
};

// Per-cell Aitken estimate of the remaining change, in units of s:
// r = d1 / d2; A = d1 r / (1 - r) / s when 0 < r < 1, else 0; clipped to +-64.
__device__ __forceinline__ double aitken_norm(double d1, double d2, double s) {
    if (d2 == 0.0) return 0.0;
    const double r = d1 / d2;
    if (!(r > 0.0 && r < 1.0)) return 0.0;
    return fmin(fmax(d1 * r / (1.0 - r) / s, -64.0), 64.0);
}

// Per-cell features from the last four temperatures (ring slots s0 = newest).
__global__ void k_accel_features(const double* __restrict__ ring, int s0, int s1, int s2, int s3, size_t Np, int n,
                                 FeatureGeom fg, __nv_bfloat16* __restrict__ x, double* __restrict__ scale) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= n) return;
    const double t0 = ring[(size_t)s0 * Np + c], t1 = ring[(size_t)s1 * Np + c];
    const double t2 = ring[(size_t)s2 * Np + c], t3 = ring[(size_t)s3 * Np + c];
    const double d1 = t0 - t1, d2 = t1 - t2, d3 = t2 - t3;
    const double s = fabs(d1) + fabs(d2) + fabs(d3) + 1e-300;
    const double V = fg.volume[c];
    double f[IN];
    f[0] = d1 / s;
    f[1] = d2 / s;
    f[2] = d3 / s;
    f[3] = aitken_norm(d1, d2, s) / 64.0;
    f[4] = fg.xspan > 0 ? (fg.centroid[3 * c] - fg.xmin) / fg.xspan : 0.0;
    f[5] = fg.yspan > 0 ? (fg.centroid[3 * c + 1] - fg.ymin) / fg.yspan : 0.0;
    f[6] = log(V / fg.vmean);
    f[7] = log10(fg.kn_num / pow(V, fg.inv_dim));
#pragma unroll
    for (int k = 0; k < IN_PAD; ++k) x[(size_t)c * IN_PAD + k] = __float2bfloat16(k < IN ? (float)f[k] : 0.0f);
    scale[c] = s;
}

// Extrapolation step.  A = the per-cell Aitken estimate (aitken_norm) and
// s = |d1| + |d2| + |d3|; learned: T = T_k + s clip(A + clip(y, +-8), +-64)
// with y the MLP's learned correction; Aitken alone: T = T_k + s A.  Then
// ebar[b][c] = C_b / Omega_tot (T - T_ref).
__global__ void k_accel_apply(const double* __restrict__ ring, int s0, int s1, int s2, size_t Np, int n,
                              const double* __restrict__ scale, const float* __restrict__ y, int learned,
                              const double* __restrict__ Cb, int n_band, double solid_angle, double T_ref,
                              double* __restrict__ T, double* __restrict__ ebar) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= n) return;
    const double t0 = ring[(size_t)s0 * Np + c];
    const double d1 = t0 - ring[(size_t)s1 * Np + c];
    const double d2 = ring[(size_t)s1 * Np + c] - ring[(size_t)s2 * Np + c];
    const double s = scale[c];
    double u = aitken_norm(d1, d2, s);
    if (learned) u = fmin(64.0, fmax(-64.0, u + fmin(8.0, fmax(-8.0, (double)y[c]))));
    const double Tn = t0 + s * u;
    T[c] = Tn;
    for (int b = 0; b < n_band; ++b) ebar[(size_t)b * Np + c] = Cb[b] / solid_angle * (Tn - T_ref);
}

// ---------------------------------------------------------------------------
// Anderson mixing of the outer iteration (accel = 3).  The source iteration
// is a fixed-point map on its state -- the cell temperatures T (which fix the
// equilibrium source) and the intensities at the cells with boundary faces
// (which the diffuse and specular walls reflect).  With the last k pairs
// (g_i = G(x_i), f_i = g_i - x_i) of state vectors the next iteration starts
// from sum_i alpha_i g_i, alpha minimising ||sum_i alpha_i f_i|| with
// sum_i alpha_i = 1 (the host solves the k x k system from the Gram matrix).
// State vector: [T (n) | e[b][d][boundary cell] * Omega_tot / C_b], the
// intensities scaled to temperature units so both parts weigh alike.

struct AaState {
    const int* bcell;  // cells with boundary faces
    int n, nbcell, n_band, n_dir;
    size_t Np;
    const double* Cb;
    double solid_angle;
    __device__ __forceinline__ size_t len() const { return (size_t)n + (size_t)n_band * n_dir * nbcell; }
    // e index and scale of state entry j >= n
    __device__ __forceinline__ size_t e_index(size_t j, double& scale) const {
        const size_t jj = j - n;
        const int i = (int)(jj % nbcell);
        const size_t bd = jj / nbcell;
        const int b = (int)(bd / n_dir), d = (int)(bd % n_dir);
        scale = solid_angle / Cb[b];
        return ((size_t)b * n_dir + d) * Np + bcell[i];
    }
};

// out = the state (T, e at the boundary cells).
__global__ void k_aa_gather(AaState a, const double* __restrict__ T, const double* __restrict__ e, double* out) {
    const size_t j = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= a.len()) return;
    if (j < (size_t)a.n) {
        out[j] = T[j];
    } else {
        double sc;
        const size_t k = a.e_index(j, sc);
        out[j] = e[k] * sc;
    }
}

constexpr int AA_MAX = 9;  // slots (depth + 1)
constexpr int AA_THREADS = 256;

struct AaMix {
    int slot[AA_MAX];  // stored slots, oldest first
    int k;
};

// The newest pair of the history: g = the state after the iteration (T, e at
// the boundary cells) written to slot `slot`, f = g - x, and the partial dot
// products f . f_s for every stored slot s (mx, the new slot included) over
// this block's grid-stride share of the state, in a fixed order:
// part[i][block] for mx.slot[i].  AA_BLOCKS blocks (a constant, so the order
// does not depend on the device).  Only the newest row of the Gram matrix is
// computed: the others do not change.
constexpr int AA_BLOCKS = 1216;
__global__ void __launch_bounds__(AA_THREADS) k_aa_push(AaState a, const double* __restrict__ T,
                                                        const double* __restrict__ e, const double* __restrict__ x,
                                                        size_t stride, int slot, AaMix mx, double* g, double* f,
                                                        double* part) {
    __shared__ double sm[AA_THREADS / 32][AA_MAX];
    const size_t len = a.len();
    double acc[AA_MAX];
#pragma unroll
    for (int i = 0; i < AA_MAX; ++i) acc[i] = 0.0;
    double* gs = g + (size_t)slot * stride;
    double* fs = f + (size_t)slot * stride;
    for (size_t j = (size_t)blockIdx.x * AA_THREADS + threadIdx.x; j < len; j += (size_t)gridDim.x * AA_THREADS) {
        double gv;
        if (j < (size_t)a.n) {
            gv = T[j];
        } else {
            double sc;
            gv = e[a.e_index(j, sc)] * sc;
        }
        const double fv = gv - x[j];
        gs[j] = gv;
        fs[j] = fv;
#pragma unroll
        for (int i = 0; i < AA_MAX; ++i)
            if (i < mx.k) acc[i] = fma(fv, mx.slot[i] == slot ? fv : f[(size_t)mx.slot[i] * stride + j], acc[i]);
    }
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
    for (int i = 0; i < AA_MAX; ++i) {
        double v = acc[i];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
        if (lane == 0) sm[warp][i] = v;
    }
    __syncthreads();
    if (threadIdx.x < AA_MAX) {
        double t = 0.0;
        for (int w = 0; w < AA_THREADS / 32; ++w) t += sm[w][threadIdx.x];
        part[(size_t)threadIdx.x * gridDim.x + blockIdx.x] = t;
    }
}

// The newest Gram row, G[slot][s] = G[s][slot] = sum over blocks of the
// partials, into the persistent slot-indexed matrix G.  One warp per stored
// slot: lane l sums blocks l, l+32, ... in order, then a fixed butterfly.
__global__ void k_aa_row(const double* __restrict__ part, int nblk, int slot, AaMix mx, double* G) {
    const int i = threadIdx.x >> 5, lane = threadIdx.x & 31;
    if (i >= mx.k) return;
    double t = 0.0;
    for (int b = lane; b < nblk; b += 32) t += part[(size_t)i * nblk + b];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) t += __shfl_xor_sync(0xffffffffu, t, o);
    if (lane == 0) {
        G[slot * AA_MAX + mx.slot[i]] = t;
        G[mx.slot[i] * AA_MAX + slot] = t;
    }
}

// One warp: alpha = G^-1 1 / (1^T G^-1 1) over the stored slots (Gram matrix
// indexed by slot, AA_MAX x AA_MAX), Tikhonov 1e-12 max(diag), Gaussian
// elimination with partial pivoting (the first row of largest |pivot|); lane
// r holds row r.  If the weights are not finite or one exceeds 1e3 the newest
// iterate is taken alone (alpha = e_k) and *flag = 1 asks the host to restart
// the history.
__global__ void k_aa_solve(const double* __restrict__ Gs, AaMix mx, double* alpha, double* flag) {
    const int lane = threadIdx.x;
    if (blockIdx.x != 0 || lane >= 32) return;
    const int k = mx.k;
    double row[AA_MAX + 1];
    double diag = 0.0;
#pragma unroll
    for (int j = 0; j <= AA_MAX; ++j) row[j] = 0.0;
    if (lane < k) {
#pragma unroll
        for (int j = 0; j < AA_MAX; ++j)
            if (j < k) row[j] = Gs[mx.slot[lane] * AA_MAX + mx.slot[j]];
#pragma unroll
        for (int j = 0; j < AA_MAX; ++j)
            if (j == lane) diag = row[j];
    }
    double dmax = diag;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) dmax = fmax(dmax, __shfl_xor_sync(0xffffffffu, dmax, o));
    bool ok = dmax > 0.0 && dmax < 1e300;
    if (lane < k) {
#pragma unroll
        for (int j = 0; j < AA_MAX; ++j)
            if (j == lane) row[j] += 1e-12 * dmax;
#pragma unroll
        for (int j = 0; j <= AA_MAX; ++j)
            if (j == k) row[j] = 1.0;
    }
#pragma unroll
    for (int c = 0; c < AA_MAX; ++c) {
        if (c >= k) break;
        // pivot: the lowest row r >= c with the largest |G[r][c]|
        double colv = 0.0;
#pragma unroll
        for (int j = 0; j < AA_MAX; ++j)
            if (j == c) colv = row[j];
        double best = (lane >= c && lane < k) ? fabs(colv) : -1.0;
        int piv = lane;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            const double ob = __shfl_xor_sync(0xffffffffu, best, o);
            const int op = __shfl_xor_sync(0xffffffffu, piv, o);
            if (ob > best || (ob == best && op < piv)) { best = ob; piv = op; }
        }
        // swap rows c and piv
#pragma unroll
        for (int j = 0; j <= AA_MAX; ++j) {
            const double vc = __shfl_sync(0xffffffffu, row[j], c);
            const double vp = __shfl_sync(0xffffffffu, row[j], piv);
            if (lane == c) row[j] = vp;
            else if (lane == piv) row[j] = vc;
        }
        double pr[AA_MAX + 1];
#pragma unroll
        for (int j = 0; j <= AA_MAX; ++j) pr[j] = __shfl_sync(0xffffffffu, row[j], c);
        double pc = 0.0;
#pragma unroll
        for (int j = 0; j < AA_MAX; ++j)
            if (j == c) pc = pr[j];
        if (pc == 0.0) ok = false;
        if (ok && lane > c && lane < k) {
            double rc = 0.0;
#pragma unroll
            for (int j = 0; j < AA_MAX; ++j)
                if (j == c) rc = row[j];
            const double f = rc / pc;
#pragma unroll
            for (int j = 0; j <= AA_MAX; ++j)
                if (j >= c) row[j] -= f * pr[j];
        }
    }
    // back substitution, row by row from the last
    double a[AA_MAX];
#pragma unroll
    for (int i = 0; i < AA_MAX; ++i) a[i] = 0.0;
    double sum = 0.0;
    if (ok) {
#pragma unroll
        for (int r = AA_MAX - 1; r >= 0; --r) {
            if (r >= k) continue;
            double rr[AA_MAX + 1];
#pragma unroll
            for (int j = 0; j <= AA_MAX; ++j) rr[j] = __shfl_sync(0xffffffffu, row[j], r);
            double v = 0.0, rk = 0.0, rd = 0.0;
#pragma unroll
            for (int j = 0; j <= AA_MAX; ++j) {
                if (j == k) rk = rr[j];
                if (j == r) rd = rr[j];
            }
            v = rk;
#pragma unroll
            for (int j = 0; j < AA_MAX; ++j)
                if (j > r && j < k) v -= rr[j] * a[j];
            a[r] = v / rd;
        }
#pragma unroll
        for (int i = 0; i < AA_MAX; ++i)
            if (i < k) sum += a[i];
#pragma unroll
        for (int i = 0; i < AA_MAX; ++i) {
            if (i < k) {
                a[i] /= sum;
                if (!(fabs(a[i]) <= 1e3)) ok = false;
            }
        }
    }
    if (lane == 0) {
        for (int i = 0; i < k; ++i) alpha[i] = ok ? a[i] : (i == k - 1 ? 1.0 : 0.0);
        *flag = ok ? 0.0 : 1.0;
    }
}

// state = sum_i alpha_i g_i: T and the boundary-cell intensities written back
// into e (the next iteration's e_prev).
__global__ void k_aa_mix(AaState a, const double* __restrict__ g, size_t stride, AaMix mx,
                         const double* __restrict__ alpha, double T_ref, double* __restrict__ T,
                         double* __restrict__ ebar, double* __restrict__ e) {
    const size_t j = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= a.len()) return;
    double t = 0.0;
    for (int i = 0; i < mx.k; ++i) t = fma(alpha[i], g[(size_t)mx.slot[i] * stride + j], t);
    if (j < (size_t)a.n) {
        T[j] = t;  // ebar follows in k_ebar_from_T
    } else {
        double sc;
        const size_t k = a.e_index(j, sc);
        e[k] = t / sc;
    }
}

// ebar[b][c] = C_b / Omega_tot (T[c] - T_ref), coalesced along the cells (grid y = band).
__global__ void k_ebar_from_T(const double* __restrict__ T, const double* __restrict__ Cb, double solid_angle,
                              double T_ref, int n, size_t Np, double* __restrict__ ebar) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    const int b = blockIdx.y;
    if (c < n) ebar[(size_t)b * Np + c] = Cb[b] / solid_angle * (T[c] - T_ref);
}

}  // namespace mlp
}  // namespace bte
