/*
 * skyr_mlp.h — C ABI of the learned multiple-scattering surrogate's network:
 * a 103 -> 64 -> 64 -> 64 -> 64 -> 3 ReLU MLP with BF16 weights and FP32
 * accumulation, its tensor-core training step (forward, relative-L2 loss,
 * backward, Adam) and batched inference.  No counterpart in the reference:
 * the network replaces the multiple-scattering heuristic of the cloud
 * raymarch (VolumetricCloudRender.comp:125-130) for order >= 2 in-scattered
 * radiance.  Conventions as in skyr.h.
 *
 * Parameter vector (FP32, the master copy the optimiser updates), layer by
 * layer, weights row-major [out][in]:
 *   W1[64][103] b1[64] W2[64][64] b2[64] W3[64][64] b3[64] W4[64][64] b4[64]
 *   W5[3][64] b5[3]                                   (19331 floats)
 *
 * Feature record (the network input, device memory): SKYR_MLP_RECORD = 112
 * bf16 values per sample, features 0..102 followed by 9 zeros (the features
 * of skyr_surrogate.h).
 *
 * Packed network (device memory, skyr_mlp_packed_bytes()): the BF16 weights
 * in padded, shared-memory-ready rows and the FP32 biases, plus the output
 * scale: prediction = output * out_scale.  It is what inference kernels read.
 */
#ifndef SKYR_MLP_H_
#define SKYR_MLP_H_

#include <stdint.h>

#include "skyr.h"

#ifdef __cplusplus
extern "C" {
#endif

#define SKYR_MLP_INPUTS 103
#define SKYR_MLP_RECORD 112
#define SKYR_MLP_WIDTH 64
#define SKYR_MLP_OUTPUTS 3
#define SKYR_MLP_PARAMS 19331

/* struct id 11 of skyr_struct_size */
typedef struct skyr_mlp_hparams {
    float learning_rate; /* Adam step size (1e-3) */
    float beta1, beta2, epsilon;
    float label_scale;   /* targets are divided by this before the loss */
    float loss_epsilon;  /* relative L2: (y - t)^2 / (y_sg^2 + loss_epsilon) */
} skyr_mlp_hparams;

int skyr_mlp_hparams_default(skyr_mlp_hparams* h);
size_t skyr_mlp_param_count(void);
size_t skyr_mlp_packed_bytes(void);

/* He-uniform weights (U(+-sqrt(6 / fan_in))) and zero biases from a seeded
 * generator, into host memory params[SKYR_MLP_PARAMS]. */
int skyr_mlp_init_params(uint64_t seed, float* params);

/* Pack FP32 parameters (device) into the packed network (device). */
int skyr_mlp_pack(skyr_ctx* ctx, const float* params, float out_scale, void* packed);

/* y[n][3] = out_scale * MLP(x[n][SKYR_MLP_RECORD]) (x bf16, y FP32, device). */
int skyr_mlp_infer(skyr_ctx* ctx, const void* packed, const uint16_t* x, int n, float* y);

/* Gradient of the mean relative-L2 loss over the n samples with respect to
 * the parameter vector (device grad[SKYR_MLP_PARAMS]) and the loss (device
 * float, may be NULL), for the network in `packed` and targets t[n][3]. */
int skyr_mlp_gradient(skyr_ctx* ctx, const void* packed, const skyr_mlp_hparams* h, const uint16_t* x,
                      const float* t, int n, float* grad, float* loss);

/* Training state: FP32 master parameters, Adam moments, the packed network. */
typedef struct skyr_mlp_trainer skyr_mlp_trainer;

int skyr_mlp_trainer_create(skyr_ctx* ctx, const float* host_params, const skyr_mlp_hparams* h,
                            skyr_mlp_trainer** out);
int skyr_mlp_trainer_destroy(skyr_mlp_trainer* tr);
/* One Adam step on the batch x[n] / t[n] (device); adds the batch loss to
 * *loss_accum (device float) when not NULL. n <= 65536. */
int skyr_mlp_train_step(skyr_mlp_trainer* tr, const uint16_t* x, const float* t, int n, float* loss_accum);
/* The full batches of one epoch without a host round trip per step: for
 * b = 0, batch, 2 batch, ... while b + batch <= n_idx, one Adam step on the
 * samples idx[b .. b + batch) of x[n_all] / t[n_all] (device; idx device
 * int32, e.g. a random permutation; the gradient kernel reads the records
 * through it, so no gathered copy is made).  An index outside [0, n_all)
 * counts as an empty sample.  Adds each step's loss to *loss_accum (device
 * float) when not NULL. */
int skyr_mlp_train_epoch(skyr_mlp_trainer* tr, const uint16_t* x, const float* t, int n_all, const int* idx,
                         int n_idx, int batch, float* loss_accum);
/* Current parameters (device FP32[SKYR_MLP_PARAMS]) and packed network. */
const float* skyr_mlp_trainer_params(const skyr_mlp_trainer* tr);
const void* skyr_mlp_trainer_packed(const skyr_mlp_trainer* tr);
int skyr_mlp_trainer_steps(const skyr_mlp_trainer* tr);
/* Change the Adam step size for the following steps (learning-rate schedules). */
int skyr_mlp_trainer_set_learning_rate(skyr_mlp_trainer* tr, float learning_rate);
/* Copy the current parameters (FP32[SKYR_MLP_PARAMS]) / packed network into
 * caller device buffers, ordered on the trainer's stream. */
int skyr_mlp_trainer_copy_params(const skyr_mlp_trainer* tr, float* out);
int skyr_mlp_trainer_copy_packed(const skyr_mlp_trainer* tr, void* out);
/* Checkpoint and resume of a training run.  save_state copies the FP32
 * parameters and both Adam moment vectors (each FP32[SKYR_MLP_PARAMS], caller
 * device buffers, ordered on the trainer's stream) and writes the step count
 * to *steps (host).  load_state replaces the trainer's parameters, moments and
 * step count with a saved state and repacks the network; the hyper-parameters
 * (learning rate included) stay the trainer's.  Training is deterministic, so
 * a run saved after k steps and resumed gives the same parameters, bit for
 * bit, as the run that went on. */
int skyr_mlp_trainer_save_state(const skyr_mlp_trainer* tr, float* params, float* m, float* v, int* steps);
int skyr_mlp_trainer_load_state(skyr_mlp_trainer* tr, const float* params, const float* m, const float* v,
                                int steps);

#ifdef __cplusplus
}
#endif
#endif /* SKYR_MLP_H_ */
