// mlp.cu — the surrogate network's training step and its C ABI: packing, the
// fixed-order reduction of the per-tile gradients with the Adam update, and
// the trainer (the tensor-core kernels of the gradient and of batched
// inference are in mlp_tc.cu).
//
// Training step = two launches:
//  1. mlp_grad_tc_kernel: one 4-warp CTA per 128 samples computes the tile's
//     loss and its partial gradient vector (forward and dZ W on tcgen05, dW on
//     the warp-level tensor path);
//  2. mlp_reduce_kernel: sums the tile partials in a fixed order
//     (deterministic), applies Adam to the FP32 master parameters and re-packs
//     the BF16 weights.
#include <cmath>
#include <cstring>
#include <new>

#include "mlp_device.cuh"
#include "skyr_ctx.cuh"

namespace skyr {
namespace mlp {

constexpr int kWarps = 4;
constexpr int kTile = 32 * kWarps;  // samples per gradient CTA (one tcgen05 M = 128 tile)
constexpr int kMaxBatch = 65536;
constexpr int kMaxBlocks = kMaxBatch / kTile;

// parameter i into the packed network (bf16 weight or f32 bias)
__device__ __forceinline__ void pack_one(unsigned char* packed, int i, float val) {
    int l = 0;
#pragma unroll 1
    while (l < kLayers - 1 && i >= b_offset(l) + fan_out(l)) ++l;
    if (i < b_offset(l)) {
        int idx = i - w_offset(l), row = idx / fan_in(l), col = idx % fan_in(l);
        reinterpret_cast<__nv_bfloat16*>(packed + packed_w_offset(l))[row * packed_stride(l) + col] =
            __float2bfloat16_rn(val);
    } else {
        reinterpret_cast<float*>(packed + kOffB)[l * kW + (i - b_offset(l))] = val;
    }
}

__global__ void __launch_bounds__(256) mlp_pack_kernel(const float* __restrict__ params, float out_scale,
                                                       unsigned char* __restrict__ packed) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < SKYR_MLP_PARAMS) pack_one(packed, i, params[i]);
    if (i == 0) *reinterpret_cast<float*>(packed + kOffScale) = out_scale;
}

// grad[i] = sum over blocks of partial[b][i] (fixed order); optional Adam
// update of params / moments and re-pack; loss: sum of the loss partials.
__global__ void __launch_bounds__(256) mlp_reduce_kernel(const float* __restrict__ partial, int nblk,
                                                         const float* __restrict__ loss_partial,
                                                         float* __restrict__ grad_out, float* __restrict__ loss_out,
                                                         int loss_accumulate, float* __restrict__ params,
                                                         float* __restrict__ m, float* __restrict__ v, float lr,
                                                         float b1, float b2, float eps, float c1, float c2,
                                                         unsigned char* __restrict__ packed) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i == 0 && loss_out) {
        float s = 0.f;
        for (int b = 0; b < nblk; ++b) s += loss_partial[b];
        *loss_out = loss_accumulate ? *loss_out + s : s;
    }
    if (i >= SKYR_MLP_PARAMS) return;
    float gsum = 0.f;
    for (int b = 0; b < nblk; ++b) gsum += partial[(size_t)b * SKYR_MLP_PARAMS + i];
    if (grad_out) grad_out[i] = gsum;
    if (params) {
        float mi = b1 * m[i] + (1.f - b1) * gsum;
        float vi = b2 * v[i] + (1.f - b2) * gsum * gsum;
        m[i] = mi;
        v[i] = vi;
        float p = params[i] - lr * (mi / c1) / (sqrtf(vi / c2) + eps);
        params[i] = p;
        pack_one(packed, i, p);
    }
}

// Batched inference on the tensor cores (mlp_tc.cu).
int launch_infer_tc(skyr_ctx* ctx, const void* packed, const uint16_t* x, int n, float* y);

int validate_hparams(const skyr_mlp_hparams* h) {
    if (!h) return set_error(SKYR_EINVAL, "null hyper-parameters");
    if (!(h->learning_rate > 0.f) || !(h->beta1 >= 0.f && h->beta1 < 1.f) || !(h->beta2 >= 0.f && h->beta2 < 1.f) ||
        !(h->epsilon > 0.f) || !(h->label_scale > 0.f) || !(h->loss_epsilon > 0.f) ||
        !std::isfinite(h->learning_rate) || !std::isfinite(h->label_scale))
        return set_error(SKYR_EINVAL, "MLP hyper-parameters out of range");
    return SKYR_OK;
}

// The gradient of one training step on the tensor cores (mlp_tc.cu).
int launch_grad_tc(skyr_ctx* ctx, const void* packed, const uint16_t* x, const float* t, const int* idx, int n_all,
                   int n, float inv_scale, float loss_eps, float* partial, float* loss_partial);

// The batch is x[idx[i]], t[idx[i]] for i < n (x[i], t[i] without idx).
int launch_grad(skyr_ctx* ctx, const void* packed, const skyr_mlp_hparams* h, const uint16_t* x, const float* t,
                const int* idx, int n_all, int n, float* partial, float* loss_partial) {
    return launch_grad_tc(ctx, packed, x, t, idx, n_all, n, 1.f / h->label_scale, h->loss_epsilon, partial,
                          loss_partial);
}

}  // namespace mlp
}  // namespace skyr

struct skyr_mlp_trainer {
    skyr_ctx* ctx = nullptr;
    skyr_mlp_hparams h{};
    float* params = nullptr;  // [P] FP32 master
    float* m = nullptr;
    float* v = nullptr;
    unsigned char* packed = nullptr;
    float* partial = nullptr;  // [kMaxBlocks][P]
    float* loss_partial = nullptr;
    int steps = 0;
};

using namespace skyr;

extern "C" {

int skyr_mlp_hparams_default(skyr_mlp_hparams* h) {
    if (!h) return set_error(SKYR_EINVAL, "null hyper-parameters");
    h->learning_rate = 1e-3f;
    h->beta1 = 0.9f;
    h->beta2 = 0.999f;
    h->epsilon = 1e-8f;
    h->label_scale = 1.f;
    h->loss_epsilon = 1e-2f;
    return SKYR_OK;
}

size_t skyr_mlp_param_count(void) { return SKYR_MLP_PARAMS; }
size_t skyr_mlp_packed_bytes(void) { return mlp::kPackedBytes; }

int skyr_mlp_init_params(uint64_t seed, float* params) {
    if (!params) return set_error(SKYR_EINVAL, "null parameters");
    // splitmix64 stream -> uniform [0, 1)
    uint64_t s = seed;
    auto next = [&]() {
        uint64_t z = (s += 0x9E3779B97F4A7C15ull);
        z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
        z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
        z ^= z >> 31;
        return (double)(z >> 11) * (1.0 / 9007199254740992.0);
    };
    for (int l = 0; l < mlp::kLayers; ++l) {
        double a = std::sqrt(6.0 / mlp::fan_in(l));
        for (int i = 0; i < mlp::fan_in(l) * mlp::fan_out(l); ++i)
            params[mlp::w_offset(l) + i] = (float)((2.0 * next() - 1.0) * a);
        for (int i = 0; i < mlp::fan_out(l); ++i) params[mlp::b_offset(l) + i] = 0.f;
    }
    return SKYR_OK;
}

int skyr_mlp_pack(skyr_ctx* ctx, const float* params, float out_scale, void* packed) {
    if (!ctx || !params || !packed) return set_error(SKYR_EINVAL, "null argument");
    if (!(out_scale > 0.f) || !std::isfinite(out_scale)) return set_error(SKYR_EINVAL, "bad output scale");
    if (int e = check_cuda(cudaSetDevice(ctx->device), "cudaSetDevice")) return e;
    if (int e = check_cuda(cudaMemsetAsync(packed, 0, mlp::kPackedBytes, ctx->stream), "clear packed network"))
        return e;
    mlp::mlp_pack_kernel<<<(SKYR_MLP_PARAMS + 255) / 256, 256, 0, ctx->stream>>>(
        params, out_scale, reinterpret_cast<unsigned char*>(packed));
    return check_cuda(cudaGetLastError(), "mlp pack kernel");
}

int skyr_mlp_infer(skyr_ctx* ctx, const void* packed, const uint16_t* x, int n, float* y) {
    if (!ctx || !packed || (n > 0 && (!x || !y))) return set_error(SKYR_EINVAL, "null argument");
    if (n < 0) return set_error(SKYR_EINVAL, "negative sample count");
    if (n == 0) return SKYR_OK;
    if ((reinterpret_cast<uintptr_t>(x) & 15) || (reinterpret_cast<uintptr_t>(packed) & 15))
        return set_error(SKYR_EINVAL, "records and packed network must be 16-byte aligned");
    if (int e = check_cuda(cudaSetDevice(ctx->device), "cudaSetDevice")) return e;
    return mlp::launch_infer_tc(ctx, packed, x, n, y);
}

int skyr_mlp_gradient(skyr_ctx* ctx, const void* packed, const skyr_mlp_hparams* h, const uint16_t* x,
                      const float* t, int n, float* grad, float* loss) {
    if (!ctx || !packed || !x || !t || !grad) return set_error(SKYR_EINVAL, "null argument");
    if (int e = mlp::validate_hparams(h)) return e;
    if (n < 1 || n > mlp::kMaxBatch) return set_error(SKYR_EINVAL, "batch size must be in [1, 65536]");
    if ((reinterpret_cast<uintptr_t>(x) & 15) || (reinterpret_cast<uintptr_t>(packed) & 15))
        return set_error(SKYR_EINVAL, "records and packed network must be 16-byte aligned");
    if (int e = check_cuda(cudaSetDevice(ctx->device), "cudaSetDevice")) return e;
    int nblk = (n + mlp::kTile - 1) / mlp::kTile;
    size_t need = ((size_t)nblk * SKYR_MLP_PARAMS + nblk) * sizeof(float);
    if (int e = ensure_pt_scratch(ctx, need)) return e;  // shared per-context scratch
    float* partial = reinterpret_cast<float*>(ctx->pt_scratch);
    float* lp = partial + (size_t)nblk * SKYR_MLP_PARAMS;
    if (int e = mlp::launch_grad(ctx, packed, h, x, t, nullptr, n, n, partial, lp)) return e;
    mlp::mlp_reduce_kernel<<<(SKYR_MLP_PARAMS + 255) / 256, 256, 0, ctx->stream>>>(
        partial, nblk, lp, grad, loss, 0, nullptr, nullptr, nullptr, 0.f, 0.f, 0.f, 0.f, 1.f, 1.f, nullptr);
    return check_cuda(cudaGetLastError(), "mlp reduce kernel");
}

int skyr_mlp_trainer_create(skyr_ctx* ctx, const float* host_params, const skyr_mlp_hparams* h,
                            skyr_mlp_trainer** out) {
    if (!ctx || !host_params || !out) return set_error(SKYR_EINVAL, "null argument");
    if (int e = mlp::validate_hparams(h)) return e;
    *out = nullptr;
    if (int e = check_cuda(cudaSetDevice(ctx->device), "cudaSetDevice")) return e;
    auto* tr = new (std::nothrow) skyr_mlp_trainer;
    if (!tr) return set_error(SKYR_ENOMEM, "out of host memory");
    tr->ctx = ctx;
    tr->h = *h;
    const size_t pb = SKYR_MLP_PARAMS * sizeof(float);
    int e = SKYR_OK;
    if (!e) e = check_cuda(cudaMalloc(&tr->params, pb), "cudaMalloc(mlp params)");
    if (!e) e = check_cuda(cudaMalloc(&tr->m, pb), "cudaMalloc(mlp m)");
    if (!e) e = check_cuda(cudaMalloc(&tr->v, pb), "cudaMalloc(mlp v)");
    if (!e) e = check_cuda(cudaMalloc(&tr->packed, mlp::kPackedBytes), "cudaMalloc(mlp packed)");
    if (!e) e = check_cuda(cudaMalloc(&tr->partial, (size_t)mlp::kMaxBlocks * pb), "cudaMalloc(mlp partials)");
    if (!e) e = check_cuda(cudaMalloc(&tr->loss_partial, mlp::kMaxBlocks * sizeof(float)), "cudaMalloc(mlp loss)");
    if (!e) e = check_cuda(cudaMemcpyAsync(tr->params, host_params, pb, cudaMemcpyHostToDevice, ctx->stream), "upload");
    if (!e) e = check_cuda(cudaMemsetAsync(tr->m, 0, pb, ctx->stream), "clear m");
    if (!e) e = check_cuda(cudaMemsetAsync(tr->v, 0, pb, ctx->stream), "clear v");
    if (!e) e = skyr_mlp_pack(ctx, tr->params, h->label_scale, tr->packed);
    if (!e) e = check_cuda(cudaStreamSynchronize(ctx->stream), "synchronize");  // host_params may go away
    if (e) {
        skyr_mlp_trainer_destroy(tr);
        return e;
    }
    *out = tr;
    return SKYR_OK;
}

int skyr_mlp_trainer_destroy(skyr_mlp_trainer* tr) {
    if (!tr) return SKYR_OK;
    if (tr->ctx) cudaSetDevice(tr->ctx->device);
    cudaFree(tr->params);
    cudaFree(tr->m);
    cudaFree(tr->v);
    cudaFree(tr->packed);
    cudaFree(tr->partial);
    cudaFree(tr->loss_partial);
    delete tr;
    return SKYR_OK;
}

namespace {
int train_step(skyr_mlp_trainer* tr, const uint16_t* x, const float* t, const int* idx, int n_all, int n,
               float* loss_accum) {
    skyr_ctx* ctx = tr->ctx;
    if (int e = mlp::launch_grad(ctx, tr->packed, &tr->h, x, t, idx, n_all, n, tr->partial, tr->loss_partial))
        return e;
    int step = tr->steps + 1;
    double c1 = 1.0 - std::pow((double)tr->h.beta1, step), c2 = 1.0 - std::pow((double)tr->h.beta2, step);
    int nblk = (n + mlp::kTile - 1) / mlp::kTile;
    mlp::mlp_reduce_kernel<<<(SKYR_MLP_PARAMS + 255) / 256, 256, 0, ctx->stream>>>(
        tr->partial, nblk, tr->loss_partial, nullptr, loss_accum, 1, tr->params, tr->m, tr->v, tr->h.learning_rate,
        tr->h.beta1, tr->h.beta2, tr->h.epsilon, (float)c1, (float)c2, tr->packed);
    if (int e = check_cuda(cudaGetLastError(), "mlp adam kernel")) return e;
    tr->steps = step;
    return SKYR_OK;
}
}  // namespace

int skyr_mlp_train_step(skyr_mlp_trainer* tr, const uint16_t* x, const float* t, int n, float* loss_accum) {
    if (!tr || !x || !t) return set_error(SKYR_EINVAL, "null argument");
    if (n < 1 || n > mlp::kMaxBatch) return set_error(SKYR_EINVAL, "batch size must be in [1, 65536]");
    if (reinterpret_cast<uintptr_t>(x) & 15) return set_error(SKYR_EINVAL, "records must be 16-byte aligned");
    if (int e = check_cuda(cudaSetDevice(tr->ctx->device), "cudaSetDevice")) return e;
    return train_step(tr, x, t, nullptr, n, n, loss_accum);
}

int skyr_mlp_train_epoch(skyr_mlp_trainer* tr, const uint16_t* x, const float* t, int n_all, const int* idx,
                         int n_idx, int batch, float* loss_accum) {
    if (!tr || !x || !t || !idx) return set_error(SKYR_EINVAL, "null argument");
    if (batch < 1 || batch > mlp::kMaxBatch) return set_error(SKYR_EINVAL, "batch size must be in [1, 65536]");
    if (n_all < 1 || n_idx < 0) return set_error(SKYR_EINVAL, "bad sample counts");
    if (reinterpret_cast<uintptr_t>(x) & 15) return set_error(SKYR_EINVAL, "records must be 16-byte aligned");
    if (int e = check_cuda(cudaSetDevice(tr->ctx->device), "cudaSetDevice")) return e;
    for (int b = 0; b + batch <= n_idx; b += batch)
        if (int e = train_step(tr, x, t, idx + b, n_all, batch, loss_accum)) return e;
    return SKYR_OK;
}
const float* skyr_mlp_trainer_params(const skyr_mlp_trainer* tr) { return tr ? tr->params : nullptr; }
const void* skyr_mlp_trainer_packed(const skyr_mlp_trainer* tr) { return tr ? tr->packed : nullptr; }
int skyr_mlp_trainer_steps(const skyr_mlp_trainer* tr) { return tr ? tr->steps : -1; }

int skyr_mlp_trainer_set_learning_rate(skyr_mlp_trainer* tr, float learning_rate) {
    if (!tr) return set_error(SKYR_EINVAL, "null trainer");
    if (!(learning_rate > 0.f) || !std::isfinite(learning_rate)) return set_error(SKYR_EINVAL, "bad learning rate");
    tr->h.learning_rate = learning_rate;
    return SKYR_OK;
}

int skyr_mlp_trainer_copy_params(const skyr_mlp_trainer* tr, float* out) {
    if (!tr || !out) return set_error(SKYR_EINVAL, "null argument");
    if (int e = check_cuda(cudaSetDevice(tr->ctx->device), "cudaSetDevice")) return e;
    return check_cuda(cudaMemcpyAsync(out, tr->params, SKYR_MLP_PARAMS * sizeof(float), cudaMemcpyDeviceToDevice,
                                      tr->ctx->stream),
                      "copy parameters");
}

int skyr_mlp_trainer_copy_packed(const skyr_mlp_trainer* tr, void* out) {
    if (!tr || !out) return set_error(SKYR_EINVAL, "null argument");
    if (int e = check_cuda(cudaSetDevice(tr->ctx->device), "cudaSetDevice")) return e;
    return check_cuda(cudaMemcpyAsync(out, tr->packed, mlp::kPackedBytes, cudaMemcpyDeviceToDevice, tr->ctx->stream),
                      "copy packed network");
}

int skyr_mlp_trainer_save_state(const skyr_mlp_trainer* tr, float* params, float* m, float* v, int* steps) {
    if (!tr || !params || !m || !v || !steps) return set_error(SKYR_EINVAL, "null argument");
    if (int e = check_cuda(cudaSetDevice(tr->ctx->device), "cudaSetDevice")) return e;
    const size_t pb = SKYR_MLP_PARAMS * sizeof(float);
    cudaStream_t st = tr->ctx->stream;
    if (int e = check_cuda(cudaMemcpyAsync(params, tr->params, pb, cudaMemcpyDeviceToDevice, st), "save parameters"))
        return e;
    if (int e = check_cuda(cudaMemcpyAsync(m, tr->m, pb, cudaMemcpyDeviceToDevice, st), "save first moments"))
        return e;
    if (int e = check_cuda(cudaMemcpyAsync(v, tr->v, pb, cudaMemcpyDeviceToDevice, st), "save second moments"))
        return e;
    *steps = tr->steps;
    return SKYR_OK;
}

int skyr_mlp_trainer_load_state(skyr_mlp_trainer* tr, const float* params, const float* m, const float* v,
                                int steps) {
    if (!tr || !params || !m || !v) return set_error(SKYR_EINVAL, "null argument");
    if (steps < 0) return set_error(SKYR_EINVAL, "negative step count");
    if (int e = check_cuda(cudaSetDevice(tr->ctx->device), "cudaSetDevice")) return e;
    const size_t pb = SKYR_MLP_PARAMS * sizeof(float);
    cudaStream_t st = tr->ctx->stream;
    if (int e = check_cuda(cudaMemcpyAsync(tr->params, params, pb, cudaMemcpyDeviceToDevice, st), "load parameters"))
        return e;
    if (int e = check_cuda(cudaMemcpyAsync(tr->m, m, pb, cudaMemcpyDeviceToDevice, st), "load first moments"))
        return e;
    if (int e = check_cuda(cudaMemcpyAsync(tr->v, v, pb, cudaMemcpyDeviceToDevice, st), "load second moments"))
        return e;
    if (int e = skyr_mlp_pack(tr->ctx, tr->params, tr->h.label_scale, tr->packed)) return e;
    tr->steps = steps;
    return SKYR_OK;
}

}  // extern "C"
