/* Learned 4x-dt time stepper for the GB300 SPH engine (libclsph_gpu.so).
 *
 * No counterpart in the reference: libclsph advances only with the plain
 * substep of sph_simulation::simulate_single_frame
 * (libclsph/sph_simulation.cpp:173-344). This interface adds
 *
 *   - a per-particle MLP (32 -> 256 -> 256 -> 4, GELU) with BF16 weights and
 *     activations and FP32 accumulation on the tensor cores, for inference and
 *     for training;
 *   - a sample collector that runs plain substeps (bit-identical to
 *     clsph_gpu_step) and records, for every substep t, the 32 neighbour
 *     features of a fixed subset of particles and the correction that would
 *     have made one 4x-dt step land where 4 plain substeps did;
 *   - the learned step: one neighbour build, density and force evaluation
 *     (the plain kernels), the MLP's acceleration correction, and one
 *     advection/collision pass over dt_mult plain time steps. The MLP also
 *     predicts the density each particle would reach under the plain solver.
 *     The next step's density pass measures the predicted density deviation
 *     of the step, max(|D - D_pred|, |M - M_pred|) over the particles with
 *     D = mean |rho/rho0 - 1| and M = mean rho/rho0 of the densities reached
 *     (rho) and predicted (rho_pred); above the threshold the step is rolled
 *     back and replaced by dt_mult plain substeps (the plain solver is both
 *     the fallback and the standard the step is measured against).
 *
 * Features of particle i (h, dt = time_delta * simulation_scale, rho0, K and
 * vmax of its scene; sums over contributing neighbours j != i,
 * d = (x_j - x_i)/h, u = (v_j - v_i) dt/h with v the particle velocity,
 * w = 1 - |d|^2; neighbour count includes i):
 *   0 rho/rho0 - 1      1 p/K          2 neighbour count / 32
 *   3-5 a dt^2/h (plain acceleration)   6-8 v' dt/h and 9 |v'|/vmax with v'
 *   the intermediate velocity
 *   10-12 sum w d       13-18 sum w d d^T (xx yy zz xy xz yz)
 *   19-21 sum w u       22-27 sum w u u^T   28 sum w d.u   29-31 sum w d x u
 * Outputs: 0-2 acceleration correction in units h/dt^2, 3 relative density
 * change over the step. Inputs and outputs are standardised with the
 * sample set's mean and standard deviation (stored with the weights);
 * standardised inputs are clamped to +-6 and, in the learned step, each
 * output to its mean +- 4 standard deviations.
 *
 * Parameter blob (floats): W1[32][256] b1[256] W2[256][256] b2[256]
 * W3[256][4] b3[4] x_mu[32] x_sigma[32] y_mu[4] y_sigma[4]; W stored
 * [input][output]. Status codes are those of clsph_gpu.h. */
#ifndef CLSPH_LEARNED_H
#define CLSPH_LEARNED_H

#include <stdint.h>

#include "clsph_gpu.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct clsph_mlp clsph_mlp;
typedef struct clsph_collector clsph_collector;

/* Number of floats in the parameter blob. */
uint64_t clsph_mlp_blob_size(void);

/* A new MLP on the current device: He-normal W1/W2 from `seed`, W3 scaled by
 * 0.01, zero biases, identity standardisation. */
int clsph_mlp_create(uint64_t seed, clsph_mlp** out);
int clsph_mlp_destroy(clsph_mlp* m);
int clsph_mlp_set_blob(clsph_mlp* m, const float* blob, uint64_t count);
int clsph_mlp_get_blob(clsph_mlp* m, float* blob, uint64_t count);

/* Fused inference on device memory: x = `rows` standardised BF16 feature rows
 * (uint16 bit patterns, [rows][32]); y = de-standardised outputs [rows][4]
 * (device floats). tcgen05 tensor cores, TMEM accumulators. Asynchronous on
 * `cuda_stream` (NULL = legacy stream); clsph_mlp_status reports a timed-out
 * tensor-core wait. */
int clsph_mlp_forward(clsph_mlp* m, const uint16_t* x_bf16, uint32_t rows, float* y, void* cuda_stream);
/* The same network on the warp-level mma.sync path (a cross-check of the
 * tcgen05 kernel). */
int clsph_mlp_forward_mma_sync(clsph_mlp* m, const uint16_t* x_bf16, uint32_t rows, float* y,
                               void* cuda_stream);
/* De-standardised predictions y_host[rows][4] (host) for raw device feature
 * rows x_raw[rows][32]. Synchronous. */
int clsph_mlp_predict(clsph_mlp* m, const float* x_raw, uint64_t rows, float* y_host);
/* Synchronises the device; *flags = error bits of clsph_mlp_forward since the
 * last call (1: a tensor-core wait timed out, 2: the final wait as well), then
 * clears them. */
int clsph_mlp_status(clsph_mlp* m, uint32_t* flags);

/* One training forward/backward pass over `rows` raw samples (device
 * x_raw[rows][32], y_raw[rows][4]) in order, without an update: writes the
 * gradients of the mean squared error of the standardised outputs (the
 * trainable part of the blob, clsph_mlp_blob_size() - 72 floats) to
 * grads_host and the loss to *loss. rows must be a multiple of 2048. */
int clsph_mlp_gradients(clsph_mlp* m, const float* x_raw, const float* y_raw, uint32_t rows,
                        float* grads_host, float* loss);

typedef struct {
  uint32_t epochs;
  uint32_t batch;        /* rows per step, a multiple of 2048 */
  float lr;              /* Adam step size at the start ... */
  float lr_final;        /* ... decaying linearly to this */
  uint64_t seed;         /* shuffling */
  int fit_normalisation; /* 1: set x/y mean and deviation from the samples first */
  uint32_t log_every;    /* steps per loss_log entry (mean loss over them) */
} clsph_train_config;

/* Adam training on device samples x_raw[samples][32], y_raw[samples][4]
 * (samples < 2^32). loss_log (may be NULL) receives up to log_len mean
 * training losses; *logged the number written. Synchronous. */
int clsph_mlp_train(clsph_mlp* m, const float* x_raw, const float* y_raw, uint64_t samples,
                    const clsph_train_config* cfg, float* loss_log, uint32_t log_len,
                    uint32_t* logged);

/* Mean standardised squared error over `samples` device samples (whole
 * 2048-row blocks only). */
int clsph_mlp_loss(clsph_mlp* m, const float* x_raw, const float* y_raw, uint64_t samples, float* loss);

/* Collector over handle h: tracks the particles whose id is a multiple of
 * id_stride and keeps up to `capacity` samples on the device. */
int clsph_collector_create(clsph_gpu* h, uint32_t id_stride, uint32_t dt_mult, uint64_t capacity,
                           clsph_collector** out);
int clsph_collector_destroy(clsph_collector* c);
/* `substeps` plain substeps of h (the same trajectory as clsph_gpu_step),
 * recording one sample per tracked particle per substep once dt_mult
 * substeps of history exist. */
int clsph_collector_step(clsph_collector* c, uint32_t substeps);
/* `steps` learned steps of h with network m (no density check), recording at
 * every visited state the samples of the plain solver's outcome from it
 * (dt_mult plain substeps from a snapshot, then back): training data from
 * the states the learned stepper itself reaches. */
int clsph_collector_step_learned(clsph_collector* c, clsph_mlp* m, uint32_t steps);
/* Device pointers to the samples so far (x [count][32], y [count][4]). */
int clsph_collector_samples(clsph_collector* c, const float** x_raw, const float** y_raw,
                            uint64_t* count);

/* Host copies of samples [first, first + count). Synchronising. */
int clsph_collector_copy(clsph_collector* c, float* x_host, float* y_host, uint64_t first, uint64_t count);

/* Raw features (float [n][32], slot order of the last sort) of the handle's
 * state after clsph_gpu_step_until(h, CLSPH_STAGE_FORCES). Synchronising;
 * for inspection and tests. */
int clsph_gpu_read_features(clsph_gpu* h, float* features_host);

typedef struct {
  uint32_t dt_mult;  /* plain time steps per learned step (4) */
  float threshold;   /* rollback when the predicted density deviation exceeds this (0.01) */
  uint32_t flags;    /* CLSPH_LEARNED_CALIBRATE: calibrate the check on fallback intervals;
                        CLSPH_LEARNED_NO_CHECK: no density check (threshold ignored) */
} clsph_learned_config;

enum { CLSPH_LEARNED_CALIBRATE = 1, CLSPH_LEARNED_NO_CHECK = 2 };

typedef struct {
  uint64_t learned_steps;  /* accepted learned steps */
  uint64_t rejected;       /* learned steps rolled back */
  uint64_t plain_substeps; /* substeps run as fallback */
  uint64_t checks;         /* density checks made */
  double deviation_sum;    /* sum of the checked predicted density deviations */
  double deviation_max;
  double particle_deviation_sum; /* sum of the checked mean |rho - rho_pred| / rho0 */
  double calibration_d;  /* current calibration of D_pred and M_pred (see below) */
  double calibration_m;
} clsph_learned_stats;

/* Advances h by `steps` x dt_mult plain time steps, each as one learned step
 * when it passes the density check, else as dt_mult plain substeps. The last
 * learned step is checked with one extra neighbour build and density pass.
 * With CLSPH_LEARNED_CALIBRATE every fallback interval also calibrates the
 * check: the plain statistics it reaches, minus those the network predicted
 * for it, update an exponential average b (weight 0.3) that is added to
 * D_pred and M_pred of later checks (the calibration belongs to the handle
 * and restarts when another network is passed). With CLSPH_LEARNED_NO_CHECK
 * the learned steps run back to back with no check, snapshot or host wait
 * (a diverging step is not caught; the call synchronises once at the end);
 * on a handle with graphs enabled (clsph_gpu_set_graph) they replay CUDA
 * graphs of 4 learned steps, with the same results.
 * stats (may be NULL) is accumulated, not cleared. */
int clsph_gpu_step_learned(clsph_gpu* h, clsph_mlp* m, uint32_t steps, const clsph_learned_config* cfg,
                           clsph_learned_stats* stats);

#ifdef __cplusplus
}
#endif

#endif
