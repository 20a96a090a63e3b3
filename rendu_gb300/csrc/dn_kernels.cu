// Denoiser kernels besides the tensor-core convolutions (dn_umma.cu): the element-wise
// pieces of a U-Net's forward and backward passes (input preparation, pooling, gradient
// routing, the ReLU and bias gradients, loss, Adam) and the fixed-order reduction of the
// weight gradient's split-K partial sums. Activations are NHWC BF16.
//
// Convolution input: up to two tensors concatenated along channels -- the first optionally
// at half resolution (nearest-neighbour 2x upsampling), the second at full resolution (the
// U-Net skip connection). With off(tap) = (tap/3 - 1, tap%3 - 1):
//   forward : out[p, co]      = act(bias[co] + sum_{tap, ci} x[p + off(tap), ci] w[tap][ci][co])
//   dgrad   : dx[p, ci]       = sum_{tap, co} g[p - off(tap), co] w[tap][ci][co]
//   wgrad   : dw[tap][ci][co] = sum_p x[p + off(tap), ci] g[p, co]
#include <cuda_bf16.h>

#include <algorithm>

#include "dn_net.hpp"

namespace rgb {
namespace dn {
namespace {

// out[i] = sum over chunks of partial[c][i], in chunk order (deterministic).
__global__ void k_reduce_chunks(const float *__restrict__ partial, int chunks, size_t n, float *__restrict__ out) {
    const size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
    if (i >= n) return;
    float s = 0.0f;
    for (int c = 0; c < chunks; ++c) s += partial[(size_t)c * n + i];
    out[i] = s;
}

// The same sum for many chunks: a block of 32 x 8 threads takes 32 consecutive outputs; thread
// row r sums chunks r, r + 8, ... (each warp reads 128 contiguous bytes per chunk), then the
// eight row sums are added in row order (deterministic).
__global__ void k_reduce_chunks_tiled(const float *__restrict__ partial, int chunks, size_t n,
                                      float *__restrict__ out) {
    __shared__ float red[8][33];
    const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;
    const size_t i = blockIdx.x * (size_t)32 + tx;
    float s = 0.0f;
    if (i < n)
        for (int c = ty; c < chunks; c += 8) s += partial[(size_t)c * n + i];
    red[ty][tx] = s;
    __syncthreads();
    if (ty == 0 && i < n) {
        float t = red[0][tx];
#pragma unroll
        for (int r = 1; r < 8; ++r) t += red[r][tx];
        out[i] = t;
    }
}

// ReLU gradient and bias-gradient partials in one pass over a (P x C) FP32 gradient, 4
// channels a thread (C a multiple of 4, C <= 1024): rows [chunk b, chunk (b + 1)) per block;
// the values of g where the forward output y was not positive (relu) count as zero; gb
// receives the masked gradient in BF16 and partial[b][c] the column sums of the masked rows
// (fixed order: per thread row by row, then thread rows 0..R-1).
__global__ void k_relu_grad_colsum4(const float *__restrict__ g, const bf16 *__restrict__ y, long P, int C, int relu,
                                    long chunk, bf16 *__restrict__ gb, float *__restrict__ partial) {
    __shared__ float4 red[256];
    const int C4 = C / 4, R = 256 / C4;
    const int r = threadIdx.x / C4, c4 = threadIdx.x % C4;
    const long pbeg = (long)blockIdx.x * chunk, pend = min(P, pbeg + chunk);
    float4 s = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    if (r < R)
        for (long p = pbeg + r; p < pend; p += R) {
            const size_t i = (size_t)p * C + 4 * c4;
            float4 v = *reinterpret_cast<const float4 *>(g + i);
            if (relu) {
                const uint2 yy = *reinterpret_cast<const uint2 *>(y + i);
                const float2 y01 = __bfloat1622float2(*reinterpret_cast<const __nv_bfloat162 *>(&yy.x));
                const float2 y23 = __bfloat1622float2(*reinterpret_cast<const __nv_bfloat162 *>(&yy.y));
                if (!(y01.x > 0.0f)) v.x = 0.0f;
                if (!(y01.y > 0.0f)) v.y = 0.0f;
                if (!(y23.x > 0.0f)) v.z = 0.0f;
                if (!(y23.y > 0.0f)) v.w = 0.0f;
            }
            const __nv_bfloat162 h01 = __floats2bfloat162_rn(v.x, v.y), h23 = __floats2bfloat162_rn(v.z, v.w);
            uint2 o;
            o.x = *reinterpret_cast<const unsigned *>(&h01);
            o.y = *reinterpret_cast<const unsigned *>(&h23);
            *reinterpret_cast<uint2 *>(gb + i) = o;
            s.x += v.x;
            s.y += v.y;
            s.z += v.z;
            s.w += v.w;
        }
    red[threadIdx.x] = s;
    __syncthreads();
    if ((int)threadIdx.x < C4) {
        float4 t = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
        for (int k = 0; k < R; ++k) {
            const float4 u = red[k * C4 + threadIdx.x];
            t.x += u.x;
            t.y += u.y;
            t.z += u.z;
            t.w += u.w;
        }
        *reinterpret_cast<float4 *>(partial + (size_t)blockIdx.x * C + 4 * threadIdx.x) = t;
    }
}

// 2x2 max pooling, NHWC.
__global__ void k_pool(const bf16 *__restrict__ x, int B, int H, int W, int C, bf16 *__restrict__ y) {
    const size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
    const int h = H / 2, w = W / 2;
    const size_t n = (size_t)B * h * w * C;
    if (i >= n) return;
    const int c = (int)(i % C);
    size_t r = i / C;
    const int xo = (int)(r % w);
    r /= w;
    const int yo = (int)(r % h);
    const int b = (int)(r / h);
    const bf16 *s = x + (((size_t)b * H + 2 * yo) * W + 2 * xo) * C + c;
    const size_t row = (size_t)W * C;
    const float m = fmaxf(fmaxf(__bfloat162float(s[0]), __bfloat162float(s[C])),
                          fmaxf(__bfloat162float(s[row]), __bfloat162float(s[row + C])));
    y[i] = __float2bfloat16_rn(m);
}

// The same, 8 channels a thread (C a multiple of 8): four 16-byte loads, one 16-byte store.
// The maximum of BF16 values is exact, so the result equals k_pool's.
__global__ void k_pool8(const bf16 *__restrict__ x, int B, int H, int W, int C, bf16 *__restrict__ y) {
    griddep_wait();  // a programmatic dependent of the convolution that wrote x
    griddep_launch();
    const size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
    const int h = H / 2, w = W / 2, c8 = C / 8;
    const size_t n = (size_t)B * h * w * c8;
    if (i >= n) return;
    const int c = (int)(i % c8) * 8;
    size_t r = i / c8;
    const int xo = (int)(r % w);
    r /= w;
    const int yo = (int)(r % h);
    const int b = (int)(r / h);
    const bf16 *s = x + (((size_t)b * H + 2 * yo) * W + 2 * xo) * C + c;
    const size_t row = (size_t)W * C;
    uint4 v[4] = {*reinterpret_cast<const uint4 *>(s), *reinterpret_cast<const uint4 *>(s + C),
                  *reinterpret_cast<const uint4 *>(s + row), *reinterpret_cast<const uint4 *>(s + row + C)};
    uint4 o;
    unsigned *ov = reinterpret_cast<unsigned *>(&o);
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        float2 m = __bfloat1622float2(reinterpret_cast<const __nv_bfloat162 *>(&v[0])[k]);
#pragma unroll
        for (int j = 1; j < 4; ++j) {
            const float2 t = __bfloat1622float2(reinterpret_cast<const __nv_bfloat162 *>(&v[j])[k]);
            m.x = fmaxf(m.x, t.x);
            m.y = fmaxf(m.y, t.y);
        }
        const __nv_bfloat162 hm = __floats2bfloat162_rn(m.x, m.y);
        ov[k] = *reinterpret_cast<const unsigned *>(&hm);
    }
    *reinterpret_cast<uint4 *>(y + (i / c8) * C + c) = o;
}

// Pooling gradient: each pooled gradient goes to the first maximal input of its window (row
// major order), added into gx. Four channels a thread (C a multiple of 4): 8-byte BF16 and
// 16-byte FP32 accesses, one read-modify-write of gx per window input that receives any.
__global__ void k_pool_back4(const bf16 *__restrict__ x, const bf16 *__restrict__ y, const float *__restrict__ gy,
                             int B, int H, int W, int C, float *__restrict__ gx) {
    const size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
    const int h = H / 2, w = W / 2, c4 = C / 4;
    const size_t n = (size_t)B * h * w * c4;
    if (i >= n) return;
    const int c = (int)(i % c4) * 4;
    size_t r = i / c4;
    const int xo = (int)(r % w);
    r /= w;
    const int yo = (int)(r % h);
    const int b = (int)(r / h);
    const size_t o = (i / c4) * C + c;  // pooled element
    const uint2 yv = *reinterpret_cast<const uint2 *>(y + o);
    const float4 g = *reinterpret_cast<const float4 *>(gy + o);
    const float2 m01 = __bfloat1622float2(*reinterpret_cast<const __nv_bfloat162 *>(&yv.x));
    const float2 m23 = __bfloat1622float2(*reinterpret_cast<const __nv_bfloat162 *>(&yv.y));
    const float m[4] = {m01.x, m01.y, m23.x, m23.y}, gv[4] = {g.x, g.y, g.z, g.w};
    const size_t base = (((size_t)b * H + 2 * yo) * W + 2 * xo) * C + c;
    const size_t row = (size_t)W * C;
    const size_t off[4] = {0, (size_t)C, row, row + C};
    unsigned done = 0u;  // channels whose gradient has been placed
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        const uint2 xv = *reinterpret_cast<const uint2 *>(x + base + off[k]);
        const float2 x01 = __bfloat1622float2(*reinterpret_cast<const __nv_bfloat162 *>(&xv.x));
        const float2 x23 = __bfloat1622float2(*reinterpret_cast<const __nv_bfloat162 *>(&xv.y));
        const float xs[4] = {x01.x, x01.y, x23.x, x23.y};
        unsigned hit = 0u;
#pragma unroll
        for (int j = 0; j < 4; ++j)
            if (!(done >> j & 1u) && xs[j] == m[j]) hit |= 1u << j;
        if (hit) {
            float4 *dst = reinterpret_cast<float4 *>(gx + base + off[k]);
            float4 v = *dst;
            if (hit & 1u) v.x += gv[0];
            if (hit & 2u) v.y += gv[1];
            if (hit & 4u) v.z += gv[2];
            if (hit & 8u) v.w += gv[3];
            *dst = v;
            done |= hit;
        }
    }
}

// Gradient of a concatenated input: channels [0, c0) go to g0 -- summed over each 2x2 block
// (the adjoint of nearest upsampling) when up0 -- and channels [c0, c0 + c1) to g1.
// Both are assigned (each is the first gradient its tensor receives). 4 channels a thread
// (c0, c1 multiples of 4): indices [0, n1) copy the skip input's channels, [n1, n1 + n0) the
// first input's (for an upsampled first input one thread per low-resolution pixel sums its
// 2 x 2 block as (a + b) + (c + d), a b / c d its pixels).
__device__ __forceinline__ float4 add4(const float4 a, const float4 b) {
    return make_float4(a.x + b.x, a.y + b.y, a.z + b.z, a.w + b.w);
}

__global__ void k_split_grad4(const float *__restrict__ gin, int B, int H, int W, int c0, int up0, int c1,
                              float *__restrict__ g0, float *__restrict__ g1) {
    const size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
    const int Cin = c0 + c1, q0 = c0 / 4, q1 = c1 / 4;
    const size_t n1 = (size_t)B * H * W * q1;
    const size_t n0 = (size_t)B * (up0 ? (H / 2) * (W / 2) : H * W) * q0;
    if (i < n1) {
        const size_t p = i / q1;
        const int c = (int)(i % q1) * 4;
        *reinterpret_cast<float4 *>(g1 + p * c1 + c) = *reinterpret_cast<const float4 *>(gin + p * Cin + c0 + c);
        return;
    }
    const size_t j = i - n1;
    if (j >= n0) return;
    const size_t p = j / q0;
    const int c = (int)(j % q0) * 4;
    if (!up0) {
        *reinterpret_cast<float4 *>(g0 + p * c0 + c) = *reinterpret_cast<const float4 *>(gin + p * Cin + c);
        return;
    }
    const int w = W / 2, h = H / 2;
    const int xl = (int)(p % w);
    const size_t r = p / w;
    const int yl = (int)(r % h);
    const int b = (int)(r / h);
    const float *s = gin + (((size_t)b * H + 2 * yl) * W + 2 * xl) * Cin + c;
    const size_t rowc = (size_t)W * Cin;
    const float4 a = *reinterpret_cast<const float4 *>(s), bb = *reinterpret_cast<const float4 *>(s + Cin);
    const float4 cc = *reinterpret_cast<const float4 *>(s + rowc), d = *reinterpret_cast<const float4 *>(s + rowc + Cin);
    *reinterpret_cast<float4 *>(g0 + p * c0 + c) = add4(add4(a, bb), add4(cc, d));
}

// Features {radiance rgb, albedo rgb, normal xyz, distance, standard error} -> 16 channels:
// log(1 + radiance), albedo, normal / 2 + 1/2, distance / (1 + distance), the relative
// standard error e = se / (luminance + 0.01) as e / (1 + e), log(1 + se), zeros; padded
// pixels replicate the nearest edge pixel.
__global__ void k_prepare(const float *__restrict__ f, int B, int H, int W, int Hp, int Wp, bf16 *__restrict__ x) {
    const size_t q = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
    const size_t n = (size_t)B * Hp * Wp;
    if (q >= n) return;
    const int xp = (int)(q % Wp);
    const size_t r = q / Wp;
    const int yp = (int)(r % Hp);
    const int b = (int)(r / Hp);
    const float *s = f + (((size_t)b * H + min(yp, H - 1)) * W + min(xp, W - 1)) * DN_FEATURES;
    float v[16];
#pragma unroll
    for (int k = 0; k < 3; ++k) v[k] = log1pf(fmaxf(s[k], 0.0f));
#pragma unroll
    for (int k = 3; k < 6; ++k) v[k] = s[k];
#pragma unroll
    for (int k = 6; k < 9; ++k) v[k] = s[k] * 0.5f + 0.5f;
    const float d = fmaxf(s[9], 0.0f);
    v[9] = d / (1.0f + d);
    const float se = fmaxf(s[10], 0.0f);
    const float lum = fmaxf(0.2126f * s[0] + 0.7152f * s[1] + 0.0722f * s[2], 0.0f);
    const float e = se / (lum + 0.01f);
    v[10] = e / (1.0f + e);
    v[11] = log1pf(se);
#pragma unroll
    for (int k = 12; k < 16; ++k) v[k] = 0.0f;
    __nv_bfloat162 o[8];
#pragma unroll
    for (int k = 0; k < 8; ++k) o[k] = __floats2bfloat162_rn(v[2 * k], v[2 * k + 1]);
    uint4 *dst = reinterpret_cast<uint4 *>(x + q * 16);
    dst[0] = *reinterpret_cast<uint4 *>(&o[0]);
    dst[1] = *reinterpret_cast<uint4 *>(&o[4]);
}

// Relative squared error, the measure the denoiser is judged by: mean over pixels and
// channels of ((x - t) / (x' + 0.01))^2 with x = dn_output(input, y) and x' the same value
// held constant (not differentiated), as in Noise2Noise's loss for Monte Carlo renders
// (Lehtinen et al. 2018): unbiased for noisy targets, which may then be independent renders
// of any sample count. dL/dy = 2 (x - t) / (x' + 0.01)^2 * (x + 1) where x > 0.
__global__ void k_relmse(const float *__restrict__ f, const float *__restrict__ y, const float *__restrict__ t, long P,
                         float *__restrict__ gy, float *__restrict__ partial) {
    __shared__ float red[256];
    const long p = blockIdx.x * (long)blockDim.x + threadIdx.x;
    float l = 0.0f;
    if (p < P) {
        const float inv = 1.0f / (3.0f * (float)P);
        const float4 yv = *reinterpret_cast<const float4 *>(y + p * 16);
        const float ys[3] = {yv.x, yv.y, yv.z};
        float g[3];
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            const float x = dn_output(f[p * DN_FEATURES + k], ys[k]);
            const float den = x + 0.01f;
            const float d = x - t[p * 3 + k];
            const float q = d / den;
            l += q * q;
            g[k] = x > 0.0f ? 2.0f * q / den * (x + 1.0f) * inv : 0.0f;
        }
        float4 *dst = reinterpret_cast<float4 *>(gy + p * 16);  // channels 3..15 carry no loss
        const float4 zero = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
        dst[0] = make_float4(g[0], g[1], g[2], 0.0f);
        dst[1] = zero;
        dst[2] = zero;
        dst[3] = zero;
    }
    red[threadIdx.x] = l;
    __syncthreads();
    for (int k = blockDim.x / 2; k > 0; k >>= 1) {
        if ((int)threadIdx.x < k) red[threadIdx.x] += red[threadIdx.x + k];
        __syncthreads();
    }
    if (threadIdx.x == 0) partial[blockIdx.x] = red[0];
}

__global__ void k_loss_total(const float *__restrict__ partial, int n, float scale, Hyper *h) {
    __shared__ float red[256];
    float s = 0.0f;
    for (int i = threadIdx.x; i < n; i += blockDim.x) s += partial[i];
    red[threadIdx.x] = s;
    __syncthreads();
    for (int k = blockDim.x / 2; k > 0; k >>= 1) {
        if ((int)threadIdx.x < k) red[threadIdx.x] += red[threadIdx.x + k];
        __syncthreads();
    }
    if (threadIdx.x == 0) h->loss = red[0] * scale;
}

__global__ void k_set_lr(Hyper *h, float lr) { h->lr = lr; }

__global__ void k_adam_step(Hyper *h) {
    const int s = h->step + 1;
    h->step = s;
    h->c1 = 1.0f - powf(h->b1, (float)s);
    h->c2 = 1.0f - powf(h->b2, (float)s);
}

// Adam (Kingma & Ba 2015) on the FP32 master parameters.
__global__ void k_adam(float *__restrict__ w, const float *__restrict__ g, float *__restrict__ m,
                       float *__restrict__ v, size_t n, const Hyper *__restrict__ h) {
    const size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float gi = g[i];
    const float mi = h->b1 * m[i] + (1.0f - h->b1) * gi;
    const float vi = h->b2 * v[i] + (1.0f - h->b2) * gi * gi;
    m[i] = mi;
    v[i] = vi;
    w[i] = w[i] - h->lr * (mi / h->c1) / (sqrtf(vi / h->c2) + h->eps);
}

inline unsigned blocks(size_t n, int t = 256) { return (unsigned)((n + t - 1) / t); }

// Rows per block of the fused ReLU / bias-gradient pass: about 2 x 152 blocks, 128 to 1,024
// rows each (a multiple of 32).
long relu_rows(long P) { return std::max(128L, std::min(1024L, (P / 304 + 31) / 32 * 32)); }

}  // namespace

// ---- launchers -------------------------------------------------------------------------------
int reduce_chunks(const float *partial, int chunks, size_t n, float *out, cudaStream_t st) {
    // Many chunks: blocks of 32 outputs x 8 chunk rows; few: a thread per output. Both orders
    // are fixed, so the result is deterministic.
    if (chunks >= 16)
        k_reduce_chunks_tiled<<<(unsigned)((n + 31) / 32), 256, 0, st>>>(partial, chunks, n, out);
    else
        k_reduce_chunks<<<blocks(n), 256, 0, st>>>(partial, chunks, n, out);
    RT_CUDA_TRY(cudaGetLastError());
    return RT_OK;
}

size_t colsum_partial_floats(long P, int C) { return (size_t)((P + relu_rows(P) - 1) / relu_rows(P)) * C; }

int pool(const bf16 *x, int B, int H, int W, int C, bf16 *y, cudaStream_t st, bool pdl) {
    if (C % 8 == 0)
        RT_CUDA_TRY(launch_pdl(k_pool8, dim3(blocks((size_t)B * (H / 2) * (W / 2) * (C / 8))), dim3(256), 0, st, pdl, x, B,
                               H, W, C, y));
    else
        k_pool<<<blocks((size_t)B * (H / 2) * (W / 2) * C), 256, 0, st>>>(x, B, H, W, C, y);
    RT_CUDA_TRY(cudaGetLastError());
    return RT_OK;
}

int pool_back(const bf16 *x, const bf16 *y, const float *gy, int B, int H, int W, int C, float *gx, cudaStream_t st) {
    if (C % 4 != 0) {
        set_error("pool_back needs a channel count that is a multiple of 4");
        return RT_ERR_ARG;
    }
    k_pool_back4<<<blocks((size_t)B * (H / 2) * (W / 2) * (C / 4)), 256, 0, st>>>(x, y, gy, B, H, W, C, gx);
    RT_CUDA_TRY(cudaGetLastError());
    return RT_OK;
}

int split_grad(const float *gin, int B, int H, int W, int c0, int up0, int c1, float *g0, float *g1, cudaStream_t st) {
    if (c0 % 4 != 0 || c1 % 4 != 0) {
        set_error("split_grad needs channel counts that are multiples of 4");
        return RT_ERR_ARG;
    }
    const size_t n = (size_t)B * H * W * (c1 / 4) + (size_t)B * (up0 ? (H / 2) * (W / 2) : H * W) * (c0 / 4);
    k_split_grad4<<<blocks(n), 256, 0, st>>>(gin, B, H, W, c0, up0, c1, g0, g1);
    RT_CUDA_TRY(cudaGetLastError());
    return RT_OK;
}

int relu_grad_bias(const float *g, const bf16 *y, long P, int C, bool relu, bf16 *gb, float *partial, float *db,
                   cudaStream_t st) {
    const long rows = relu_rows(P);
    const int chunks = (int)((P + rows - 1) / rows);
    if (C % 4 != 0 || C > 1024) {
        set_error("relu_grad_bias needs a channel count that is a multiple of 4, at most 1024");
        return RT_ERR_ARG;
    }
    k_relu_grad_colsum4<<<chunks, 256, 0, st>>>(g, y, P, C, relu ? 1 : 0, rows, gb, partial);
    RT_CUDA_TRY(cudaGetLastError());
    return reduce_chunks(partial, chunks, (size_t)C, db, st);
}

int prepare(const float *f, int B, int H, int W, int Hp, int Wp, bf16 *x, cudaStream_t st) {
    k_prepare<<<blocks((size_t)B * Hp * Wp), 256, 0, st>>>(f, B, H, W, Hp, Wp, x);
    RT_CUDA_TRY(cudaGetLastError());
    return RT_OK;
}

int relmse_loss(const float *f, const float *y, const float *target, long P, float *gy, float *partial, Hyper *hyper,
                cudaStream_t st) {
    const unsigned nb = blocks((size_t)P);
    k_relmse<<<nb, 256, 0, st>>>(f, y, target, P, gy, partial);
    k_loss_total<<<1, 256, 0, st>>>(partial, (int)nb, 1.0f / (3.0f * (float)P), hyper);
    RT_CUDA_TRY(cudaGetLastError());
    return RT_OK;
}

int set_learning_rate(Hyper *hyper, float lr, cudaStream_t st) {
    k_set_lr<<<1, 1, 0, st>>>(hyper, lr);
    RT_CUDA_TRY(cudaGetLastError());
    return RT_OK;
}

int adam(float *params, const float *grads, float *m, float *v, size_t n, Hyper *hyper, cudaStream_t st) {
    k_adam_step<<<1, 1, 0, st>>>(hyper);
    k_adam<<<blocks(n), 256, 0, st>>>(params, grads, m, v, n, hyper);
    RT_CUDA_TRY(cudaGetLastError());
    return RT_OK;
}

}  // namespace dn
}  // namespace rgb
