// Denoiser: a 5-level U-Net over NHWC BF16 activations, trained and run with the kernels of
// dn_kernels.cu. Shared declarations of the kernel launchers and the network state.
#pragma once

#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <cstdint>
#include <vector>

#include "rt_context.hpp"

namespace rgb {
namespace dn {

using bf16 = __nv_bfloat16;

// Input of a 3x3 convolution: channels [0, c0) from p0, read at half resolution when up0
// (nearest-neighbour 2x upsampling), then channels [c0, c0 + c1) from p1 at full resolution.
// c0 and c1 are multiples of 8; all tensors are NHWC with 16-byte aligned bases.
struct ConvIn {
    const bf16 *p0 = nullptr;
    int c0 = 0;
    int up0 = 0;
    const bf16 *p1 = nullptr;
    int c1 = 0;
};

// Per-layer weight table entry for the fused Adam update (offsets into the flat buffers).
struct LayerW {
    uint32_t woff, cin, cout;
};
constexpr int kMaxLayers = 24;
struct LayerTable {
    LayerW l[kMaxLayers];
    int n;
};

// Hyper-parameters in device memory, so that a captured update can be replayed.
struct Hyper {
    float lr, b1, b2, eps;
    float c1, c2;  // bias corrections 1 - b^step
    int step;
    float loss;
};

// ---- launchers (asynchronous on st; RT_OK or RT_ERR_CUDA) -------------------------------------
// out[p, co] = act(bias[co] + sum_{tap, ci} in[p + off(tap), ci] * w[tap][ci][co]); K = 9 (c0 + c1).
int conv_forward(const ConvIn &in, int B, int H, int W, const bf16 *w, const float *bias, int Cout, bool relu,
                 bf16 *out_bf, float *out_f, cudaStream_t st);
// dw[tap][ci][co] = sum_p in[p + off(tap), ci] * g[p, co]; partial holds wgrad_partial_floats().
int conv_wgrad(const ConvIn &in, int B, int H, int W, const bf16 *g, int Cout, float *partial, float *dw,
               cudaStream_t st);
size_t wgrad_partial_floats(long P, int Cin, int Cout);
// db[c] = sum_p g[p, c]; partial holds colsum_partial_floats().
int colsum(const float *g, long P, int C, float *partial, float *db, cudaStream_t st);
size_t colsum_partial_floats(long P, int C);
// wt[8 - tap][co][ci] = bf16(w[tap][ci][co]) (dgrad weights), wb = bf16(w).
int convert_weights(const float *w, int Cin, int Cout, bf16 *wb, bf16 *wt, cudaStream_t st);
int pool(const bf16 *x, int B, int H, int W, int C, bf16 *y, cudaStream_t st);
int pool_back(const bf16 *x, const bf16 *y, const float *gy, int B, int H, int W, int C, float *gx, cudaStream_t st);
int split_grad(const float *gin, int B, int H, int W, int c0, int up0, int c1, float *g0, float *g1, cudaStream_t st);
// g = relu ? g * (y > 0) : g (in place), gb = bf16(g).
int relu_grad(float *g, const bf16 *y, size_t n, bool relu, bf16 *gb, cudaStream_t st);
// Features (B, H, W, 10) fp32 -> network input (B, Hp, Wp, 16) bf16, edge-replicated padding.
int prepare(const float *f, int B, int H, int W, int Hp, int Wp, bf16 *x, cudaStream_t st);
// Network output (B, Hp, Wp, 16) fp32 + input log radiance -> radiance (B, H, W, 3).
int finish(const bf16 *x, const float *y, int B, int H, int W, int Hp, int Wp, float *out, cudaStream_t st);
// Loss in log space on the residual prediction; writes gy (P x 16) and hyper->loss.
int l1_loss(const bf16 *x, const float *y, const float *target, long P, float *gy, float *partial, Hyper *hyper,
            cudaStream_t st);
int adam(float *params, const float *grads, float *m, float *v, size_t n, const LayerTable &tab, Hyper *hyper,
         bf16 *wb, bf16 *wt, cudaStream_t st);

}  // namespace dn
}  // namespace rgb
