// C-ABI of the learned denoiser (include/rendu_gb300.h, dn_*): the U-Net's layer graph, its
// activation and gradient buffers, the forward and backward passes over the kernels of
// dn_kernels.cu, and the Adam update.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include "dn_net.hpp"

using namespace rgb;
using namespace rgb::dn;

namespace {

struct DeviceGuard {
    int prev = -1;
    explicit DeviceGuard(int dev) {
        cudaGetDevice(&prev);
        if (prev != dev) cudaSetDevice(dev);
    }
    ~DeviceGuard() {
        int cur = -1;
        cudaGetDevice(&cur);
        if (prev >= 0 && cur != prev) cudaSetDevice(prev);
    }
};

int arg_error(const char *msg) {
    set_error(msg);
    return RT_ERR_ARG;
}

struct Tensor {
    int level;  // resolution divided by 2^level
    int ch;
    bool f32;   // FP32 (network output) instead of BF16
};

struct Conv {
    int src0, up0, src1;  // tensor indices (src1 = -1: no skip input)
    int cin0, cin1, cout;
    int relu;
    int out;
    size_t woff, boff;        // FP32 weights and bias in the flat parameters
    size_t wk_off, wkd_off;   // packed forward / data-gradient BF16 weights
};

struct Op {
    bool pool;
    int conv;      // index into convs (when !pool)
    int src, out;  // tensors of a pooling op
};

constexpr int kLevels = 5;
constexpr int kChannels[kLevels] = {32, 48, 64, 96, 128};
constexpr int kInC = 16, kOutC = 16;

size_t align_up(size_t x, size_t a) { return (x + a - 1) / a * a; }

// What a captured step depends on: the shape and every buffer address baked into it.
struct GraphSig {
    const void *p[11];
    int B, H, W, Hp, Wp;
};

// One captured step: the first call with a new signature runs eagerly (and configures
// the kernels), the second captures, later ones replay.
struct GraphSlot {
    cudaGraphExec_t exec = nullptr;
    GraphSig sig{};
    bool seen = false;
};

}  // namespace

struct dn_net {
    int device = 0;
    cudaStream_t stream = nullptr;  // for host-pointer calls
    // The weight gradients run on a second stream beside the data-gradient chain (forked
    // and joined with events, captured into the same graph).
    cudaStream_t side = nullptr;
    cudaEvent_t ev_fork = nullptr, ev_join = nullptr;
    std::vector<Tensor> tensors;
    std::vector<Conv> convs;
    std::vector<Op> ops;
    size_t nparams = 0;
    PackTable table{};
    DevBuf params, grads, adam_m, adam_v, wk, wkd, hyper;  // wk, wkd: packed BF16 weight copies
    float lr_dev = -1.0f;  // learning rate held in device memory
    // Shape-dependent buffers.
    int B = 0, Hp = 0, Wp = 0;
    bool train_ready = false;
    DevBuf act, gact, gin, gbf, partial, bpartial, feat, target, out, loss_partial, ups;
    std::vector<size_t> act_off, gact_off, gb_off;  // gb_off: per convolution, its BF16 output gradient
    GraphSlot g_train, g_infer;

    bf16 *bf(int t) { return reinterpret_cast<bf16 *>(static_cast<char *>(act.ptr) + act_off[t]); }
    float *f(int t) { return reinterpret_cast<float *>(static_cast<char *>(act.ptr) + act_off[t]); }
    float *g(int t) { return reinterpret_cast<float *>(static_cast<char *>(gact.ptr) + gact_off[t]); }
    bf16 *gb(size_t conv) { return reinterpret_cast<bf16 *>(static_cast<char *>(gbf.ptr) + gb_off[conv]); }
    Hyper *hyp() { return hyper.as<Hyper>(); }
    long pixels(int level) const { return (long)B * (Hp >> level) * (Wp >> level); }
};

namespace {

// The U-Net: per level two 3x3 convolutions + ReLU (32, 48, 64, 96, 128 channels) with 2x2
// max pooling between levels; on the way up, each level's first convolution reads the
// level below upsampled 2x concatenated with the skip tensor of its own level; a final
// convolution to 16 channels (no ReLU, FP32).
void build_graph(dn_net *n) {
    auto tensor = [&](int level, int ch, bool f32) {
        n->tensors.push_back({level, ch, f32});
        return (int)n->tensors.size() - 1;
    };
    auto conv = [&](int s0, int up0, int s1, int cout, int relu, bool f32) {
        Conv c;
        c.src0 = s0;
        c.up0 = up0;
        c.src1 = s1;
        c.cin0 = n->tensors[s0].ch;
        c.cin1 = s1 >= 0 ? n->tensors[s1].ch : 0;
        c.cout = cout;
        c.relu = relu;
        const int level = n->tensors[s0].level - (up0 ? 1 : 0);
        c.out = tensor(level, cout, f32);
        c.woff = n->nparams;
        n->nparams += (size_t)9 * (c.cin0 + c.cin1) * cout;
        c.boff = n->nparams;
        n->nparams += cout;
        n->convs.push_back(c);
        n->ops.push_back({false, (int)n->convs.size() - 1, -1, -1});
        return c.out;
    };
    auto pool_op = [&](int s) {
        const int o = tensor(n->tensors[s].level + 1, n->tensors[s].ch, false);
        n->ops.push_back({true, -1, s, o});
        return o;
    };
    int cur = tensor(0, kInC, false);
    int skip[kLevels];
    for (int l = 0; l < kLevels; ++l) {
        if (l) cur = pool_op(cur);
        cur = conv(cur, 0, -1, kChannels[l], 1, false);
        cur = conv(cur, 0, -1, kChannels[l], 1, false);
        skip[l] = cur;
    }
    for (int l = kLevels - 2; l >= 0; --l) {
        cur = conv(cur, 1, skip[l], kChannels[l], 1, false);
        cur = conv(cur, 0, -1, kChannels[l], 1, false);
    }
    conv(cur, 0, -1, kOutC, 0, true);
    n->table.n = (int)n->convs.size();
    uint64_t fo = 0, bo = 0;
    for (size_t i = 0; i < n->convs.size(); ++i) {
        Conv &c = n->convs[i];
        c.wk_off = fo;
        c.wkd_off = bo;
        n->table.e[i] = {(uint32_t)c.woff, (uint32_t)c.cin0, (uint32_t)c.cin1, (uint32_t)c.cout, fo, bo};
        fo += (uint64_t)c.cout * packed_k(c.cin0, c.cin1);
        bo += (uint64_t)(c.cin0 + c.cin1) * packed_k(c.cout, 0);
    }
    n->table.fwd_total = fo;
    n->table.bwd_total = bo;
}

// Packed BF16 forward and data-gradient copies of every layer's weights.
int refresh_weights(dn_net *n, cudaStream_t st) {
    return pack_all(n->params.as<float>(), n->table, n->wk.as<bf16>(), n->wkd.as<bf16>(), st);
}

int reset_optimizer(dn_net *n, cudaStream_t st) {
    RT_CUDA_TRY(cudaMemsetAsync(n->adam_m.ptr, 0, n->nparams * sizeof(float), st));
    RT_CUDA_TRY(cudaMemsetAsync(n->adam_v.ptr, 0, n->nparams * sizeof(float), st));
    RT_CUDA_TRY(cudaMemsetAsync(n->grads.ptr, 0, n->nparams * sizeof(float), st));
    const Hyper h{1e-3f, 0.9f, 0.999f, 1e-8f, 1.0f, 1.0f, 0, 0.0f};
    RT_CUDA_TRY(cudaMemcpyAsync(n->hyper.ptr, &h, sizeof(Hyper), cudaMemcpyHostToDevice, st));
    n->lr_dev = h.lr;
    return RT_OK;
}

int upload_params(dn_net *n, const float *host, cudaStream_t st) {
    RT_CUDA_TRY(cudaMemcpyAsync(n->params.ptr, host, n->nparams * sizeof(float), cudaMemcpyHostToDevice, st));
    int r = refresh_weights(n, st);
    if (r == RT_OK) r = reset_optimizer(n, st);
    if (r == RT_OK) RT_CUDA_TRY(cudaStreamSynchronize(st));
    return r;
}

// He-normal weights (std sqrt(2 / fan_in), the last layer scaled by 0.1 so that the
// network starts close to the identity on its noisy input), zero biases. splitmix64 +
// Box-Muller: deterministic for a seed on every platform.
std::vector<float> he_init(const dn_net *n, uint64_t seed) {
    std::vector<float> h(n->nparams, 0.0f);
    uint64_t s = seed ^ 0x6A09E667F3BCC909ull;
    auto next = [&]() {
        s += 0x9E3779B97F4A7C15ull;
        uint64_t z = s;
        z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
        z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
        return z ^ (z >> 31);
    };
    auto unif = [&]() { return ((double)(next() >> 11) + 0.5) * (1.0 / 9007199254740992.0); };
    for (size_t li = 0; li < n->convs.size(); ++li) {
        const Conv &c = n->convs[li];
        const size_t nw = (size_t)9 * (c.cin0 + c.cin1) * c.cout;
        double sd = std::sqrt(2.0 / (9.0 * (c.cin0 + c.cin1)));
        if (li + 1 == n->convs.size()) sd *= 0.1;
        for (size_t i = 0; i < nw; ++i) {
            const double u1 = unif(), u2 = unif();
            h[c.woff + i] = (float)(sd * std::sqrt(-2.0 * std::log(u1)) * std::cos(6.283185307179586 * u2));
        }
    }
    return h;
}

int ensure_shape(dn_net *n, int B, int Hp, int Wp, bool train) {
    if (n->B == B && n->Hp == Hp && n->Wp == Wp && (!train || n->train_ready)) return RT_OK;
    n->B = B;
    n->Hp = Hp;
    n->Wp = Wp;
    n->act_off.assign(n->tensors.size(), 0);
    n->gact_off.assign(n->tensors.size(), 0);
    size_t a = 0, g = 0, gbytes = 0, max_gin = 0, max_part = 0, max_bpart = 0, max_ups = 0;
    for (size_t t = 0; t < n->tensors.size(); ++t) {
        const Tensor &T = n->tensors[t];
        const size_t el = (size_t)n->pixels(T.level) * T.ch;
        n->act_off[t] = a;
        a += align_up(el * (T.f32 ? 4 : 2), 256);
        n->gact_off[t] = g;
        g += align_up(el * 4, 256);
    }
    n->gb_off.assign(n->convs.size(), 0);
    for (size_t i = 0; i < n->convs.size(); ++i) {
        const Conv &c = n->convs[i];
        const long P = n->pixels(n->tensors[c.out].level);
        const int cin = c.cin0 + c.cin1;
        if (c.cin1 || c.up0) max_gin = std::max(max_gin, (size_t)P * cin);
        if (c.up0) max_ups = std::max(max_ups, (size_t)P * c.cin0);
        max_part = std::max(max_part, wgrad_partial_floats(P, cin, c.cout));
        max_bpart = std::max(max_bpart, colsum_partial_floats(P, c.cout));
        n->gb_off[i] = gbytes;
        gbytes += align_up((size_t)P * c.cout * 2, 256);
    }
    if (n->act.reserve(a) != RT_OK || n->ups.reserve(std::max<size_t>(max_ups, 8) * 2) != RT_OK) return RT_ERR_OOM;
    n->train_ready = false;
    if (train) {
        const long P0 = n->pixels(0);
        if (n->gact.reserve(g) != RT_OK || n->gin.reserve(std::max<size_t>(max_gin, 1) * 4) != RT_OK ||
            n->gbf.reserve(gbytes) != RT_OK || n->partial.reserve(max_part * 4) != RT_OK ||
            n->bpartial.reserve(max_bpart * 4) != RT_OK ||
            n->loss_partial.reserve((size_t)((P0 + 255) / 256) * 4) != RT_OK)
            return RT_ERR_OOM;
        n->train_ready = true;
    }
    return RT_OK;
}

// The forward pass; the output layer stores its FP32 result (for the loss), or with
// last.finish_out writes the denoised image instead.
int forward(dn_net *n, cudaStream_t st, const FOut &last) {
    for (const Op &op : n->ops) {
        int r;
        if (op.pool) {
            const Tensor &s = n->tensors[op.src];
            r = pool(n->bf(op.src), n->B, n->Hp >> s.level, n->Wp >> s.level, s.ch, n->bf(op.out), st, true);
        } else {
            const Conv &c = n->convs[op.conv];
            const Tensor &o = n->tensors[c.out];
            ConvIn in;
            in.p0 = n->bf(c.src0);
            in.c0 = c.cin0;
            in.up0 = c.up0;
            in.p1 = c.src1 >= 0 ? n->bf(c.src1) : nullptr;
            in.c1 = c.cin1;
            r = conv_forward_umma(in, n->B, n->Hp >> o.level, n->Wp >> o.level, n->wk.as<bf16>() + c.wk_off,
                                  n->params.as<float>() + c.boff, c.cout, c.relu != 0, o.f32 ? nullptr : n->bf(c.out),
                                  o.f32 && !last.finish_out ? n->f(c.out) : nullptr, n->ups.as<bf16>(), st,
                                  o.f32 ? last : FOut(), true);
        }
        if (r != RT_OK) return r;
    }
    return RT_OK;
}

// The backward pass. Per convolution: the ReLU mask and bias gradient give the BF16 output
// gradient (a buffer per convolution); the data gradient follows on `st` (the critical
// chain), the weight gradient on the side stream, which waits for the output gradient and
// rejoins `st` at the end. Each branch has its own split-K scratch (bias partials on `st`,
// weight partials and the upsampled input on the side stream).
int backward(dn_net *n, const float *target, cudaStream_t st) {
    const int last = n->convs.back().out;
    int r = relmse_loss(n->feat.as<float>(), n->f(last), target, n->pixels(0), n->g(last), n->loss_partial.as<float>(),
                        n->hyp(), st);
    if (r != RT_OK) return r;
    float *grads = n->grads.as<float>();
    bool forked = false;
    for (auto it = n->ops.rbegin(); it != n->ops.rend() && r == RT_OK; ++it) {
        const Op &op = *it;
        if (op.pool) {
            const Tensor &s = n->tensors[op.src];
            r = pool_back(n->bf(op.src), n->bf(op.out), n->g(op.out), n->B, n->Hp >> s.level, n->Wp >> s.level, s.ch,
                          n->g(op.src), st);
            continue;
        }
        const Conv &c = n->convs[op.conv];
        const Tensor &o = n->tensors[c.out];
        const int H = n->Hp >> o.level, W = n->Wp >> o.level;
        const long P = n->pixels(o.level);
        bf16 *gb = n->gb(op.conv);
        r = relu_grad_bias(n->g(c.out), c.relu ? n->bf(c.out) : nullptr, P, c.cout, c.relu != 0, gb,
                           n->bpartial.as<float>(), grads + c.boff, st);
        if (r != RT_OK) break;
        cudaError_t e = cudaEventRecord(n->ev_fork, st);
        if (e == cudaSuccess) e = cudaStreamWaitEvent(n->side, n->ev_fork, 0);
        if (e != cudaSuccess) {
            set_error(std::string("denoiser stream fork failed: ") + cudaGetErrorString(e));
            r = RT_ERR_CUDA;
            break;
        }
        forked = true;
        ConvIn in;
        in.p0 = n->bf(c.src0);
        in.c0 = c.cin0;
        in.up0 = c.up0;
        in.p1 = c.src1 >= 0 ? n->bf(c.src1) : nullptr;
        in.c1 = c.cin1;
        r = conv_wgrad(in, n->B, H, W, gb, c.cout, n->partial.as<float>(), grads + c.woff, n->ups.as<bf16>(), n->side);
        if (r != RT_OK || c.src0 == 0) continue;  // no gradient for the network input
        ConvIn gi;
        gi.p0 = gb;
        gi.c0 = c.cout;
        const bool split = c.cin1 || c.up0;
        float *dst = split ? n->gin.as<float>() : n->g(c.src0);
        r = conv_forward_umma(gi, n->B, H, W, n->wkd.as<bf16>() + c.wkd_off, nullptr, c.cin0 + c.cin1, false, nullptr,
                              dst, nullptr, st, FOut(), true);
        if (r == RT_OK && split)
            r = split_grad(dst, n->B, H, W, c.cin0, c.up0, c.cin1, n->g(c.src0), c.src1 >= 0 ? n->g(c.src1) : nullptr,
                           st);
    }
    // Rejoin on every path, so that a capture always ends with one stream.
    if (forked) {
        cudaError_t e = cudaEventRecord(n->ev_join, n->side);
        if (e == cudaSuccess) e = cudaStreamWaitEvent(st, n->ev_join, 0);
        if (e != cudaSuccess && r == RT_OK) {
            set_error(std::string("denoiser stream join failed: ") + cudaGetErrorString(e));
            r = RT_ERR_CUDA;
        }
    }
    return r;
}

bool aligned16(const void *p) { return ((uintptr_t)p & 15u) == 0; }


int check_train_shape(const float *features, const float *target, uint32_t width, uint32_t height, uint32_t batch) {
    if (!features || !target || width == 0 || height == 0 || batch == 0) return arg_error("empty denoiser batch");
    if (width % 16 || height % 16) return arg_error("training crops must be multiples of 16 pixels wide and high");
    if ((uint64_t)width * height * batch >= (1ull << 31)) return arg_error("denoiser batch too large");
    return RT_OK;
}

// Copy a caller's array (host, or device with dev) into an internal buffer.
int stage(DevBuf &buf, const float *src, size_t n, bool dev, cudaStream_t st) {
    if (buf.reserve(n * sizeof(float)) != RT_OK) return RT_ERR_OOM;
    RT_CUDA_TRY(cudaMemcpyAsync(buf.ptr, src, n * sizeof(float), dev ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice,
                                st));
    return RT_OK;
}

int set_lr(dn_net *n, float lr, cudaStream_t st) {
    if (!(lr >= 0.0f) || !std::isfinite(lr)) return arg_error("learning rate must be finite and >= 0");
    if (lr != n->lr_dev) {
        const int r = set_learning_rate(n->hyp(), lr, st);
        if (r != RT_OK) return r;
        n->lr_dev = lr;
    }
    return RT_OK;
}

int adam_launch(dn_net *n, cudaStream_t st) {
    const int r = adam(n->params.as<float>(), n->grads.as<float>(), n->adam_m.as<float>(), n->adam_v.as<float>(),
                       n->nparams, n->hyp(), st);
    return r == RT_OK ? refresh_weights(n, st) : r;
}

// Forward + loss + backward over the staged batch in n->feat / n->target.
int train_body(dn_net *n, bool with_adam, cudaStream_t st) {
    int r = prepare(n->feat.as<float>(), n->B, n->Hp, n->Wp, n->Hp, n->Wp, n->bf(0), st);
    if (r == RT_OK) r = forward(n, st, FOut());
    if (r == RT_OK) r = backward(n, n->target.as<float>(), st);
    if (r == RT_OK && with_adam) r = adam_launch(n, st);
    return r;
}

GraphSig signature(dn_net *n, int H, int W) {
    GraphSig g;
    std::memset(&g, 0, sizeof(g));
    const DevBuf *bufs[11] = {&n->act, &n->gact, &n->gin, &n->gbf, &n->partial, &n->bpartial, &n->feat, &n->target,
                              &n->out, &n->loss_partial, &n->ups};
    for (int i = 0; i < 11; ++i) g.p[i] = bufs[i]->ptr;
    g.B = n->B;
    g.H = H;
    g.W = W;
    g.Hp = n->Hp;
    g.Wp = n->Wp;
    return g;
}

template <class Body>
int run_graph(dn_net *n, GraphSlot &slot, const GraphSig &sig, Body body, cudaStream_t st) {
    if (!slot.seen || std::memcmp(&slot.sig, &sig, sizeof(GraphSig)) != 0) {
        if (slot.exec) cudaGraphExecDestroy(slot.exec);
        slot.exec = nullptr;
        slot.sig = sig;
        slot.seen = true;
        return body(st);
    }
    if (!slot.exec) {
        RT_CUDA_TRY(cudaStreamBeginCapture(n->stream, cudaStreamCaptureModeThreadLocal));
        const int r = body(n->stream);
        cudaGraph_t g = nullptr;
        const cudaError_t e = cudaStreamEndCapture(n->stream, &g);
        cudaError_t ei = cudaSuccess;
        if (r == RT_OK && e == cudaSuccess) ei = cudaGraphInstantiate(&slot.exec, g, cudaGraphInstantiateFlagUseNodePriority);
        if (g) cudaGraphDestroy(g);
        if (r != RT_OK || e != cudaSuccess || ei != cudaSuccess) {
            slot.exec = nullptr;
            slot.seen = false;
            cudaGetLastError();
            if (r != RT_OK) return r;
            set_error(std::string("denoiser graph capture failed: ") + cudaGetErrorString(e != cudaSuccess ? e : ei));
            return RT_ERR_CUDA;
        }
    }
    RT_CUDA_TRY(cudaGraphLaunch(slot.exec, st));
    return RT_OK;
}

int stage_batch(dn_net *n, const float *features, const float *target, uint32_t width, uint32_t height,
                uint32_t batch, bool dev, cudaStream_t st) {
    int r = check_train_shape(features, target, width, height, batch);
    if (r == RT_OK) r = ensure_shape(n, (int)batch, (int)height, (int)width, true);
    const size_t np = (size_t)batch * height * width;
    if (r == RT_OK) r = stage(n->feat, features, np * DN_FEATURES, dev, st);
    if (r == RT_OK) r = stage(n->target, target, np * 3, dev, st);
    return r;
}

int read_loss(dn_net *n, float *loss, cudaStream_t st) {
    if (!loss) return RT_OK;
    RT_CUDA_TRY(cudaMemcpyAsync(loss, &n->hyp()->loss, sizeof(float), cudaMemcpyDeviceToHost, st));
    RT_CUDA_TRY(cudaStreamSynchronize(st));
    return umma_status(true);
}

int finish_host_call(cudaStream_t st) {
    RT_CUDA_TRY(cudaStreamSynchronize(st));
    return umma_status(true);
}

}  // namespace

extern "C" {

RT_API int dn_create(dn_net **out, int device) {
    if (!out) return arg_error("null output handle");
    *out = nullptr;
    int count = 0;
    if (cudaGetDeviceCount(&count) != cudaSuccess || device < 0 || device >= count) {
        cudaGetLastError();
        set_error("CUDA device " + std::to_string(device) + " is not available");
        return RT_ERR_CUDA;
    }
    DeviceGuard guard(device);
    dn_net *n = new dn_net();
    n->device = device;
    build_graph(n);
    int r = RT_OK;
    // The data-gradient chain is the critical path of a training step: its stream gets the
    // highest priority, the weight-gradient stream the lowest (captured into the graphs'
    // kernel nodes, which are instantiated to use them).
    int prio_lo = 0, prio_hi = 0;
    cudaDeviceGetStreamPriorityRange(&prio_lo, &prio_hi);
    if (cudaStreamCreateWithPriority(&n->stream, cudaStreamNonBlocking, prio_hi) != cudaSuccess ||
        cudaStreamCreateWithPriority(&n->side, cudaStreamNonBlocking, prio_lo) != cudaSuccess ||
        cudaEventCreateWithFlags(&n->ev_fork, cudaEventDisableTiming) != cudaSuccess ||
        cudaEventCreateWithFlags(&n->ev_join, cudaEventDisableTiming) != cudaSuccess) {
        cudaGetLastError();
        set_error("stream creation failed");
        r = RT_ERR_CUDA;
    }
    const size_t pb = n->nparams * sizeof(float);
    if (r == RT_OK &&
        (n->params.reserve(pb) != RT_OK || n->grads.reserve(pb) != RT_OK || n->adam_m.reserve(pb) != RT_OK ||
         n->adam_v.reserve(pb) != RT_OK || n->wk.reserve(n->table.fwd_total * 2) != RT_OK ||
         n->wkd.reserve(n->table.bwd_total * 2) != RT_OK || n->hyper.reserve(sizeof(Hyper)) != RT_OK))
        r = RT_ERR_OOM;
    if (r == RT_OK) {
        const std::vector<float> h = he_init(n, 0);
        r = upload_params(n, h.data(), n->stream);
    }
    if (r != RT_OK) {
        dn_destroy(n);
        return r;
    }
    clear_error();
    *out = n;
    return RT_OK;
}

RT_API int dn_destroy(dn_net *n) {
    if (!n) return RT_OK;
    DeviceGuard guard(n->device);
    if (n->stream) cudaStreamSynchronize(n->stream);
    if (n->side) cudaStreamSynchronize(n->side);
    for (GraphSlot *g : {&n->g_train, &n->g_infer})
        if (g->exec) cudaGraphExecDestroy(g->exec);
    for (DevBuf *b : {&n->params, &n->grads, &n->adam_m, &n->adam_v, &n->wk, &n->wkd, &n->hyper, &n->act, &n->gact,
                      &n->gin, &n->gbf, &n->partial, &n->bpartial, &n->feat, &n->target, &n->out, &n->loss_partial,
                      &n->ups})
        b->release();
    if (n->ev_fork) cudaEventDestroy(n->ev_fork);
    if (n->ev_join) cudaEventDestroy(n->ev_join);
    if (n->side) cudaStreamDestroy(n->side);
    if (n->stream) cudaStreamDestroy(n->stream);
    delete n;
    return RT_OK;
}

RT_API int dn_init(dn_net *n, uint64_t seed) {
    if (!n) return arg_error("null network");
    DeviceGuard guard(n->device);
    const std::vector<float> h = he_init(n, seed);
    return upload_params(n, h.data(), n->stream);
}

RT_API int dn_layer_count(const dn_net *n, uint32_t *count) {
    if (!n || !count) return arg_error("null argument");
    *count = (uint32_t)n->convs.size();
    return RT_OK;
}

RT_API int dn_layer_info(const dn_net *n, uint32_t layer, dn_layer *out) {
    if (!n || !out) return arg_error("null argument");
    if (layer >= n->convs.size()) return arg_error("layer index out of range");
    const Conv &c = n->convs[layer];
    out->cin0 = (uint32_t)c.cin0;
    out->cin1 = (uint32_t)c.cin1;
    out->cout = (uint32_t)c.cout;
    out->up0 = c.up0;
    out->relu = c.relu;
    out->level = n->tensors[c.out].level;
    out->weight_offset = c.woff;
    out->bias_offset = c.boff;
    return RT_OK;
}

RT_API int dn_param_count(const dn_net *n, size_t *count) {
    if (!n || !count) return arg_error("null argument");
    *count = n->nparams;
    return RT_OK;
}

RT_API int dn_get_params(dn_net *n, float *out, size_t count) {
    if (!n || !out || count != n->nparams) return arg_error("parameter count mismatch");
    DeviceGuard guard(n->device);
    RT_CUDA_TRY(cudaDeviceSynchronize());
    RT_CUDA_TRY(cudaMemcpy(out, n->params.ptr, count * sizeof(float), cudaMemcpyDeviceToHost));
    return umma_status(true);
}

RT_API int dn_set_params(dn_net *n, const float *in, size_t count) {
    if (!n || !in || count != n->nparams) return arg_error("parameter count mismatch");
    DeviceGuard guard(n->device);
    RT_CUDA_TRY(cudaDeviceSynchronize());
    return upload_params(n, in, n->stream);
}

RT_API int dn_get_grads(dn_net *n, float *out, size_t count) {
    if (!n || !out || count != n->nparams) return arg_error("parameter count mismatch");
    DeviceGuard guard(n->device);
    RT_CUDA_TRY(cudaDeviceSynchronize());
    RT_CUDA_TRY(cudaMemcpy(out, n->grads.ptr, count * sizeof(float), cudaMemcpyDeviceToHost));
    return umma_status(true);
}

RT_API int dn_read_grads(dn_net *n, float *out, size_t count, void *stream, uint32_t flags) {
    if (!n || !out || count != n->nparams) return arg_error("parameter count mismatch");
    DeviceGuard guard(n->device);
    if (flags & RT_FLAG_DEVICE_PTRS) {
        RT_CUDA_TRY(cudaMemcpyAsync(out, n->grads.ptr, count * sizeof(float), cudaMemcpyDeviceToDevice,
                                    static_cast<cudaStream_t>(stream)));
        return RT_OK;
    }
    return dn_get_grads(n, out, count);
}

RT_API int dn_write_grads(dn_net *n, const float *in, size_t count, void *stream, uint32_t flags) {
    if (!n || !in || count != n->nparams) return arg_error("parameter count mismatch");
    DeviceGuard guard(n->device);
    if (flags & RT_FLAG_DEVICE_PTRS) {
        RT_CUDA_TRY(cudaMemcpyAsync(n->grads.ptr, in, count * sizeof(float), cudaMemcpyDeviceToDevice,
                                    static_cast<cudaStream_t>(stream)));
        return RT_OK;
    }
    RT_CUDA_TRY(cudaDeviceSynchronize());
    RT_CUDA_TRY(cudaMemcpy(n->grads.ptr, in, count * sizeof(float), cudaMemcpyHostToDevice));
    return RT_OK;
}

RT_API int dn_denoise(dn_net *n, const float *features, uint32_t width, uint32_t height, uint32_t batch, float *out,
                      void *stream, uint32_t flags) {
    if (!n || !features || !out) return arg_error("null argument");
    if (width == 0 || height == 0 || batch == 0) return arg_error("empty image");
    const uint32_t Hp = (height + 15) / 16 * 16, Wp = (width + 15) / 16 * 16;
    if ((uint64_t)Wp * Hp * batch >= (1ull << 31)) return arg_error("image too large");
    DeviceGuard guard(n->device);
    const bool dev = (flags & RT_FLAG_DEVICE_PTRS) != 0;
    cudaStream_t st = dev ? static_cast<cudaStream_t>(stream) : n->stream;
    int r = ensure_shape(n, (int)batch, (int)Hp, (int)Wp, false);
    const size_t np = (size_t)batch * height * width;
    if (r == RT_OK) r = stage(n->feat, features, np * DN_FEATURES, dev, st);
    if (r == RT_OK && n->out.reserve(np * 3 * sizeof(float)) != RT_OK) r = RT_ERR_OOM;
    if (r != RT_OK) return r;
    const int B = (int)batch, H = (int)height, W = (int)width;
    auto body = [&](cudaStream_t s) {
        FOut fin;
        fin.feat = n->feat.as<float>();
        fin.finish_out = n->out.as<float>();
        fin.H = H;
        fin.W = W;
        int q = prepare(n->feat.as<float>(), B, H, W, (int)Hp, (int)Wp, n->bf(0), s);
        if (q == RT_OK) q = forward(n, s, fin);
        return q;
    };
    r = run_graph(n, n->g_infer, signature(n, H, W), body, st);
    if (r != RT_OK) return r;
    RT_CUDA_TRY(cudaMemcpyAsync(out, n->out.ptr, np * 3 * sizeof(float),
                                dev ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost, st));
    return dev ? RT_OK : finish_host_call(st);
}

RT_API int dn_backward(dn_net *n, const float *features, const float *target, uint32_t width, uint32_t height,
                       uint32_t batch, float *loss, void *stream, uint32_t flags) {
    if (!n) return arg_error("null network");
    DeviceGuard guard(n->device);
    const bool dev = (flags & RT_FLAG_DEVICE_PTRS) != 0;
    cudaStream_t st = dev ? static_cast<cudaStream_t>(stream) : n->stream;
    int r = stage_batch(n, features, target, width, height, batch, dev, st);
    if (r == RT_OK) r = train_body(n, false, st);
    if (r == RT_OK) r = read_loss(n, loss, st);
    if (r == RT_OK && !dev) r = finish_host_call(st);
    return r;
}

RT_API int dn_adam_step(dn_net *n, float lr, void *stream) {
    if (!n) return arg_error("null network");
    DeviceGuard guard(n->device);
    cudaStream_t st = stream ? static_cast<cudaStream_t>(stream) : n->stream;
    // NULL: the network's own stream, after everything already queued on the device (the
    // gradients may have been written on the legacy default stream, which the network's
    // non-blocking stream does not wait for), and the call blocks.
    if (!stream) RT_CUDA_TRY(cudaDeviceSynchronize());
    int r = set_lr(n, lr, st);
    if (r == RT_OK) r = adam_launch(n, st);
    if (r == RT_OK && !stream) RT_CUDA_TRY(cudaStreamSynchronize(st));
    return r;
}

RT_API int dn_train_step(dn_net *n, const float *features, const float *target, uint32_t width, uint32_t height,
                         uint32_t batch, float lr, float *loss, void *stream, uint32_t flags) {
    if (!n) return arg_error("null network");
    DeviceGuard guard(n->device);
    const bool dev = (flags & RT_FLAG_DEVICE_PTRS) != 0;
    cudaStream_t st = dev ? static_cast<cudaStream_t>(stream) : n->stream;
    int r = set_lr(n, lr, st);
    if (r == RT_OK) r = stage_batch(n, features, target, width, height, batch, dev, st);
    if (r == RT_OK)
        r = run_graph(n, n->g_train, signature(n, (int)height, (int)width),
                      [&](cudaStream_t s) { return train_body(n, true, s); }, st);
    if (r == RT_OK) r = read_loss(n, loss, st);
    if (r == RT_OK && !dev) r = finish_host_call(st);
    return r;
}

RT_API int dn_conv3x3(const void *x0, uint32_t c0, int32_t up0, const void *x1, uint32_t c1, uint32_t batch,
                      uint32_t height, uint32_t width, const void *weights, const float *bias, uint32_t cout,
                      int32_t relu, void *out, int32_t out_fp32, void *stream) {
    if (!x0 || !weights || !out || (c1 && !x1)) return arg_error("null argument");
    if (c0 == 0 || c0 % 8 || c1 % 8 || cout == 0 || cout % 8) return arg_error("channel counts must be multiples of 8");
    if (batch == 0 || height == 0 || width == 0) return arg_error("empty input");
    if (up0 && (height % 2 || width % 2)) return arg_error("an upsampled input needs an even output size");
    if (!aligned16(x0) || (x1 && !aligned16(x1)) || !aligned16(weights))
        return arg_error("inputs and weights must be 16-byte aligned");
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    void *wk = nullptr, *ups = nullptr;
    RT_CUDA_TRY(cudaMallocAsync(&wk, (size_t)cout * packed_k((int)c0, (int)c1) * sizeof(bf16), st));
    if (up0 && cudaMallocAsync(&ups, (size_t)batch * height * width * c0 * sizeof(bf16), st) != cudaSuccess) {
        cudaGetLastError();
        cudaFreeAsync(wk, st);
        set_error("scratch allocation failed");
        return RT_ERR_OOM;
    }
    int r = pack_weights_bf16(static_cast<const bf16 *>(weights), (int)c0, (int)c1, (int)cout, static_cast<bf16 *>(wk),
                              st);
    if (r == RT_OK) {
        ConvIn in;
        in.p0 = static_cast<const bf16 *>(x0);
        in.c0 = (int)c0;
        in.up0 = up0 ? 1 : 0;
        in.p1 = static_cast<const bf16 *>(x1);
        in.c1 = (int)c1;
        r = conv_forward_umma(in, (int)batch, (int)height, (int)width, static_cast<const bf16 *>(wk), bias, (int)cout,
                              relu != 0, out_fp32 ? nullptr : static_cast<bf16 *>(out),
                              out_fp32 ? static_cast<float *>(out) : nullptr, static_cast<bf16 *>(ups), st);
    }
    cudaFreeAsync(wk, st);
    if (ups) cudaFreeAsync(ups, st);
    return r;
}

RT_API int dn_conv3x3_backward(const void *x0, uint32_t c0, int32_t up0, const void *x1, uint32_t c1, uint32_t batch,
                               uint32_t height, uint32_t width, const float *weights, uint32_t cout, const void *gy,
                               float *dx, float *dw, void *stream) {
    if (!x0 || !gy || (c1 && !x1) || (dx && !weights)) return arg_error("null argument");
    if (c0 == 0 || c0 % 8 || c1 % 8 || cout == 0 || cout % 8) return arg_error("channel counts must be multiples of 8");
    if (batch == 0 || height == 0 || width == 0) return arg_error("empty input");
    if (up0 && (height % 2 || width % 2)) return arg_error("an upsampled input needs an even output size");
    if (!aligned16(x0) || (x1 && !aligned16(x1)) || !aligned16(gy)) return arg_error("inputs must be 16-byte aligned");
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    const int cin = (int)(c0 + c1);
    const long P = (long)batch * height * width;
    int r = RT_OK;
    if (dx) {
        void *wkd = nullptr;
        RT_CUDA_TRY(cudaMallocAsync(&wkd, (size_t)cin * packed_k((int)cout, 0) * sizeof(bf16), st));
        r = pack_weights(weights, (int)c0, (int)c1, (int)cout, nullptr, static_cast<bf16 *>(wkd), st);
        if (r == RT_OK) {
            ConvIn gi;
            gi.p0 = static_cast<const bf16 *>(gy);
            gi.c0 = (int)cout;
            r = conv_forward_umma(gi, (int)batch, (int)height, (int)width, static_cast<const bf16 *>(wkd), nullptr, cin,
                                  false, nullptr, dx, nullptr, st);
        }
        cudaFreeAsync(wkd, st);
        if (r != RT_OK) return r;
    }
    if (dw) {
        void *part = nullptr, *ups = nullptr;
        RT_CUDA_TRY(cudaMallocAsync(&part, wgrad_partial_floats(P, cin, (int)cout) * sizeof(float), st));
        if (up0) RT_CUDA_TRY(cudaMallocAsync(&ups, (size_t)P * c0 * sizeof(bf16), st));
        ConvIn in;
        in.p0 = static_cast<const bf16 *>(x0);
        in.c0 = (int)c0;
        in.up0 = up0 ? 1 : 0;
        in.p1 = static_cast<const bf16 *>(x1);
        in.c1 = (int)c1;
        r = conv_wgrad(in, (int)batch, (int)height, (int)width, static_cast<const bf16 *>(gy), (int)cout,
                       static_cast<float *>(part), dw, static_cast<bf16 *>(ups), st);
        cudaFreeAsync(part, st);
        if (ups) cudaFreeAsync(ups, st);
    }
    return r;
}

}  // extern "C"
