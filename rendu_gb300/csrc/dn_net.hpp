// Denoiser: a 5-level U-Net over NHWC BF16 activations, trained and run with the kernels of
// dn_kernels.cu. Shared declarations of the kernel launchers and the network state.
#pragma once

#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <cstdint>
#include <utility>
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

// Per-layer entry of the weight-packing table: FP32 parameters at woff, packed forward
// weights at fwd_off (Cout x packed_k(c0, c1)), packed data-gradient weights at bwd_off
// ((c0 + c1) x packed_k(Cout, 0)).
constexpr int kMaxLayers = 24;
struct PackEntry {
    uint32_t woff, c0, c1, cout;
    uint64_t fwd_off, bwd_off;
};
struct PackTable {
    PackEntry e[kMaxLayers];
    int n;
    uint64_t fwd_total, bwd_total;
};

// Hyper-parameters in device memory, so that a captured update can be replayed.
struct Hyper {
    float lr, b1, b2, eps;
    float c1, c2;  // bias corrections 1 - b^step
    int step;
    float loss;
};

// radiance = max(exp(log(1 + input) + y) - 1, 0): the network predicts a correction of the
// noisy input in log space; the input is taken from the FP32 features, so that a zero
// correction returns the input unchanged.
__device__ __forceinline__ float dn_output(float in, float y) { return fmaxf(expm1f(log1pf(fmaxf(in, 0.0f)) + y), 0.0f); }

// The output layer's result finished in its epilogue (conv_forward_umma's `fo`, inference):
// instead of storing the FP32 output, each pixel of the H x W image inside the padded grid
// writes the denoised radiance finish_out[o, k] = dn_output(feat[o, k], y[k]), k < 3, o its
// index in the image (Cout a multiple of 16).
struct FOut {
    const float *feat = nullptr;  // (B, H, W, DN_FEATURES)
    float *finish_out = nullptr;  // (B, H, W, 3)
    int H = 0, W = 0;
};

// Programmatic dependent launch: a kernel launched with the programmatic-serialisation
// attribute (launch_pdl with pdl) may start while the kernel before it on the stream
// finishes; griddep_wait() blocks until that kernel has completed and its writes are
// visible (at once without the attribute), griddep_launch() lets the next such kernel start.
__device__ __forceinline__ void griddep_wait() { asm volatile("griddepcontrol.wait;\n" ::: "memory"); }
__device__ __forceinline__ void griddep_launch() { asm volatile("griddepcontrol.launch_dependents;\n" ::: "memory"); }

template <class... P, class... A>
cudaError_t launch_pdl(void (*kernel)(P...), dim3 grid, dim3 block, size_t smem, cudaStream_t st, bool pdl,
                       A &&...args) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = grid;
    cfg.blockDim = block;
    cfg.dynamicSmemBytes = smem;
    cfg.stream = st;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = attr;
    cfg.numAttrs = pdl ? 1 : 0;
    return cudaLaunchKernelEx(&cfg, kernel, std::forward<A>(args)...);
}

// ---- launchers (asynchronous on st; RT_OK or RT_ERR_CUDA) -------------------------------------
// Length of a packed weight row: 9 taps x (64-channel chunks of input 0 + of input 1) x 64.
size_t packed_k(int c0, int c1);
// Tensor-core convolution (dn_umma.cu): out[p, co] = act(bias[co] + sum_{tap, ci}
// in[p + off(tap), ci] w[tap][ci][co]) with the weights packed by pack_weights; with the
// data-gradient packing it computes a layer's input gradient. An upsampled input 0 is
// first expanded into `ups` (B x H x W x c0 BF16). Cout a multiple of 8.
// pdl: launch as a programmatic dependent of the previous kernel on st (its prologue reads
// the weights and bias before waiting for that kernel, so they must not come from it: the
// network's own packed weights, not a caller's freshly written buffers).
int conv_forward_umma(const ConvIn &in, int B, int H, int W, const bf16 *wpk, const float *bias, int Cout, bool relu,
                      bf16 *out_bf, float *out_f, bf16 *ups, cudaStream_t st, const FOut &fo = FOut(),
                      bool pdl = false);
// w FP32 [tap][c0 + c1][Cout] -> wpk [Cout][packed_k(c0, c1)] (forward) and
// wpkd [c0 + c1][packed_k(Cout, 0)] (data gradient, taps mirrored); either may be null.
int pack_weights(const float *w, int c0, int c1, int Cout, bf16 *wpk, bf16 *wpkd, cudaStream_t st);
int pack_weights_bf16(const bf16 *w, int c0, int c1, int Cout, bf16 *wpk, cudaStream_t st);
// Both packings of every layer in the table, from the flat FP32 parameters.
int pack_all(const float *params, const PackTable &tab, bf16 *wk, bf16 *wkd, cudaStream_t st);
// RT_ERR_TIMEOUT if a tensor-core convolution's bounded wait gave up (synchronous).
int umma_status(bool clear);
// dw[tap][ci][co] = sum_p in[p + off(tap), ci] * g[p, co] on the tensor cores (dn_umma.cu);
// partial holds wgrad_partial_floats() floats; an upsampled input 0 is first expanded into
// `ups` (B x H x W x c0 BF16).
int conv_wgrad(const ConvIn &in, int B, int H, int W, const bf16 *g, int Cout, float *partial, float *dw, bf16 *ups,
               cudaStream_t st);
size_t wgrad_partial_floats(long P, int Cin, int Cout);
// out[i] = sum_{c < chunks} partial[c n + i], in chunk order.
int reduce_chunks(const float *partial, int chunks, size_t n, float *out, cudaStream_t st);
// Scratch floats of relu_grad_bias's bias-gradient partials.
size_t colsum_partial_floats(long P, int C);
int pool(const bf16 *x, int B, int H, int W, int C, bf16 *y, cudaStream_t st, bool pdl = false);
int pool_back(const bf16 *x, const bf16 *y, const float *gy, int B, int H, int W, int C, float *gx, cudaStream_t st);
int split_grad(const float *gin, int B, int H, int W, int c0, int up0, int c1, float *g0, float *g1, cudaStream_t st);
// The ReLU gradient (g with zeros where the forward output y was not positive, as a BF16 copy
// in gb; g itself is left as it is) and the bias gradient db[c] = sum over the P rows of the
// masked g, in one pass (partial: colsum_partial_floats(P, C) floats of scratch).
int relu_grad_bias(const float *g, const bf16 *y, long P, int C, bool relu, bf16 *gb, float *partial, float *db,
                   cudaStream_t st);
// Features (B, H, W, DN_FEATURES) fp32 -> network input (B, Hp, Wp, 16) bf16, edge-replicated
// padding.
int prepare(const float *f, int B, int H, int W, int Hp, int Wp, bf16 *x, cudaStream_t st);
// Relative squared error of the output (y: P x 16) against the target (P pixels, features
// and output at the same P); writes gy (P x 16) and hyper->loss.
int relmse_loss(const float *f, const float *y, const float *target, long P, float *gy, float *partial, Hyper *hyper,
                cudaStream_t st);
// hyper->lr = lr, ordered on st (the value travels as a kernel argument: no host buffer).
int set_learning_rate(Hyper *hyper, float lr, cudaStream_t st);
// Adam on the FP32 parameters (the packed BF16 copies are refreshed by pack_all).
int adam(float *params, const float *grads, float *m, float *v, size_t n, Hyper *hyper, cudaStream_t st);

}  // namespace dn
}  // namespace rgb
