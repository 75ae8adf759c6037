/*
 * fastscape_surrogate.h -- C ABI of the learned surrogate that jumps
 * FastScape realizations many timesteps ahead, and of the judged ensemble
 * that alternates its jumps with the plain FP64 timestep.
 *
 * The reference has no learned part: everything here is added beside the
 * plain timestep (fastscape_RB.cpp:366-373), which generates the training
 * data, judges the jumps and takes over where a jump is not good enough.
 *
 * The network is a 4-level convolutional encoder-decoder over a
 * realization's whole grid: per level two 3x3 convolutions with ReLU
 * (channels c, 2c, 4c, 8c with c = base_channels), 2x2 average pooling down,
 * nearest-neighbour upsampling concatenated with the encoder's output of the
 * same level on the way up, and a 1x1 output head. Inputs are 16 planes: the
 * elevation divided by s = max(max h, u), log(s/u)/4, K, m and U mapped to
 * about [-1, 1], the ring mask, log2 of the drainage count / 16 (from an
 * erosion-free analysis of the field: receivers, ordering, accumulation),
 * and on cells with a full neighbourhood the drop to the D8 receiver, the
 * central differences along x and y (times 1/2) and h minus 1/8 of the sum
 * of its 8 neighbours, each divided by u; the last five planes are zero.
 * u = jump*U*dt is the uplift of one jump. It predicts
 * y = (h_{t+jump} - h_t)/u on interior cells; rings never change. Activations and weights are BF16, products accumulate in FP32 on
 * the tensor cores (tcgen05), the master weights and Adam's moments are
 * FP32. Training minimises the mean over samples of
 *   (u / relief_{t+jump})^2 * mean over interior cells of (y_pred - y)^2,
 * the squared elevation error of the jump relative to the relief it reaches
 * (relief = max h - min h = max h: the rings stay at 0).
 *
 * Every function returns FS_OK or a negative FS_ERR_* status
 * (fs_last_error() holds the text), like include/fastscape_gb300.h.
 */
#ifndef FASTSCAPE_SURROGATE_H
#define FASTSCAPE_SURROGATE_H

#include "fastscape_gb300.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct fs_surrogate fs_surrogate;

typedef struct fs_sg_config {
  int width, height;   /* grid of every realization the network takes: 128 to
                          4096, multiples of 64 (each of the four levels must
                          tile in 128-pixel blocks)                          */
  int base_channels;   /* c: 32 (channels 32..256, ~1.95M parameters) or 16  */
  int batch;           /* training batch, and samples per inference pass     */
  int jump;            /* timesteps one prediction spans                     */
  double dt;           /* timestep of the realizations (yr)                  */
  uint64_t seed;       /* weight initialisation and batch sampling           */
} fs_sg_config;

/* 512 x 512, c = 32, batch 32, jump 50, dt 1000, seed 1. */
void fs_sg_config_default(fs_sg_config *c);

fs_surrogate *fs_sg_create(const fs_sg_config *c, int *status);
void fs_sg_destroy(fs_surrogate *s);
int fs_sg_get_config(const fs_surrogate *s, fs_sg_config *c);

/* Parameters as one FP32 vector: per convolution layer (14, in forward
 * order) the weights [cout][tap][cin] (tap = 3*dy + dx) then the biases
 * [cout], then the head's weights [c] and bias. */
int fs_sg_param_count(const fs_surrogate *s, int64_t *n);
int fs_sg_get_params(const fs_surrogate *s, float *out);
int fs_sg_set_params(fs_surrogate *s, const float *in);
/* Gradients of the last training step, same layout. */
int fs_sg_get_grads(const fs_surrogate *s, float *out);
/* Parameters to / from a file (config checked on load). */
int fs_sg_save(const fs_surrogate *s, const char *path);
int fs_sg_load(fs_surrogate *s, const char *path);

/* ---- data ---------------------------------------------------------------
 * Samples live on the device: h_t (FP32), the target y (FP32) and per-sample
 * constants. fs_sg_reserve sets the capacity (it discards the samples). */
int fs_sg_reserve(fs_surrogate *s, int capacity);
/* Appends n samples from host fields: h_t[k], h_next[k] (width*height
 * doubles each, h_next = h_t advanced `jump` timesteps) and params[k]. */
int fs_sg_add_samples(fs_surrogate *s, int n, const double *h_t, const double *h_next,
                      const fs_params *params);
/* Generates samples on the GPU with the plain batched method: ntraj
 * realizations from seeded uniform [0,1) noise (rings 0) with K, m, U drawn
 * as in the ragged ensemble (K log-uniform [1e-6, 1e-5], m uniform
 * [0.3, 0.6], U log-uniform [1e-4, 5e-3], n 1, dx 100); realization r
 * records per_traj samples at timesteps t = o_r + k*max_spinup/per_traj
 * (o_r a random multiple of 10 below that spacing, so t is spread over
 * [0, max_spinup)), each (h_t, h_{t+jump}). *added = samples appended. */
int fs_sg_generate(fs_surrogate *s, int ntraj, int per_traj, int max_spinup, uint64_t seed,
                   int *added);
/* The last `held` samples form the held-out split (default 0). */
int fs_sg_set_holdout(fs_surrogate *s, int held);
int fs_sg_dataset_info(const fs_surrogate *s, int *nsamples, int *held);
/* Copies sample k back (h_t and target y, width*height floats each; either
 * may be NULL). */
int fs_sg_get_sample(const fs_surrogate *s, int k, float *h_t, float *y);

/* ---- training -----------------------------------------------------------
 * `steps` Adam steps (b1 0.9, b2 0.999, eps 1e-8, learning rate lr) on
 * batches drawn uniformly from the training split; *mean_loss = the mean
 * training loss over those steps. */
int fs_sg_train(fs_surrogate *s, int steps, float lr, double *mean_loss);
/* Mean loss over the held-out split (or over all samples when none is held
 * out), without updating anything. */
int fs_sg_eval(fs_surrogate *s, double *loss);
/* The same loss for the two jumps that need no network, over the same
 * samples: uplift only (y_pred = 1: h + u on interior cells, erosion
 * ignored) and no change (y_pred = 0). What the trained network gains over
 * the method without it is its loss against these. */
int fs_sg_eval_baselines(fs_surrogate *s, double *uplift_only, double *no_change);
/* One forward/backward pass on samples idx[0..n) (n <= batch), leaving the
 * gradients for fs_sg_get_grads; no update. */
int fs_sg_grad(fs_surrogate *s, int n, const int *idx, double *loss);
/* Device time of the last fs_sg_train call (ms) and the tensor-core
 * convolutions' FLOPs of one training step (forward, data and weight
 * gradients). */
int fs_sg_train_stats(const fs_surrogate *s, double *ms, double *conv_flops_per_step);

/* ---- inference ----------------------------------------------------------
 * Jumps n fields h_in (host, width*height doubles each) with their params:
 * h_out = h_in + u*y_pred on interior cells, rings unchanged. */
int fs_sg_predict_host(fs_surrogate *s, int n, const double *h_in, const fs_params *params,
                       double *h_out);
/* Jumps realizations idx[0..n) of batch b (same grid as the network) in
 * place on the device; when d_out is not NULL, writes realization idx[k]'s
 * jump to the device field d_out[k] instead. Ordered against the batch's
 * stream; returns when the fields are written. */
int fs_sg_predict_batch(fs_surrogate *s, fs_batch *b, int n, const int *idx,
                        double *const *d_out);
/* Device time (CUDA events on the network's stream) of one forward pass
 * over a full batch of dataset samples -- input planes, the fourteen
 * convolutions, pooling and concatenation -- averaged over `reps` passes
 * after one warm-up, and the convolutions' FLOPs of that pass. */
int fs_sg_time_forward(fs_surrogate *s, int reps, double *ms_per_pass, double *flops_per_pass);
/* FLOPs of the convolutions of one inference pass over one realization. */
int fs_sg_infer_flops(const fs_surrogate *s, double *flops);

/* ---- judged ensemble ----------------------------------------------------
 * Advances every realization of batch b by nsteps timesteps, alternating a
 * surrogate jump (`jump` timesteps) with plain_steps plain FP64 timesteps
 * per cycle (timesteps left over at the end run plain). In every cycle a
 * seeded judge_fraction of the realizations still on the surrogate has its
 * jump re-run exactly (`jump` plain timesteps from the same state): the
 * relief-normalised RMS elevation error RMS(h_jump - h_exact)/relief(h_exact)
 * over interior cells and the receiver agreement (share of interior cells
 * whose D8 receiver is the same in both fields) are measured, the exact
 * field is kept, and a realization whose error exceeds max_rel_rms or whose
 * agreement falls below min_agreement runs the plain timestep for the rest
 * of the run. */
typedef struct fs_sg_ensemble_opts {
  int nsteps;
  int plain_steps;         /* plain timesteps after each jump (1)           */
  double judge_fraction;   /* 0.05                                          */
  double max_rel_rms;      /* 0.01                                          */
  double min_agreement;    /* 0.99                                          */
  uint64_t seed;           /* which jumps are judged                        */
} fs_sg_ensemble_opts;

typedef struct fs_sg_ensemble_stats {
  int cycles, jumps, judged, fallbacks;
  double rel_rms_mean, rel_rms_max, agreement_mean, agreement_min;
  double ms_total, ms_infer, ms_exact, ms_plain, ms_judge;  /* host clock  */
  /* the judge's measures for the field before the jump (no change) against
   * the exact run, over the same judged jumps: how far the landscape and
   * its receivers move in one jump */
  double rel_rms_unchanged_mean, agreement_unchanged_mean;
} fs_sg_ensemble_stats;

void fs_sg_ensemble_defaults(fs_sg_ensemble_opts *o);

/* The judge's measures for n host field pairs (width*height doubles each; a
 * = candidate, b = exact, params[k] gives the neighbour distances):
 * rel_rms[k] = RMS over interior cells of (a - b) / (max b - min b), and
 * agreement[k] = share of interior cells whose D8 receiver (the reference's
 * order and tie-break, fastscape_RB.cpp:160-182) is the same in a and b. */
int fs_sg_compare_host(int width, int height, const fs_params *params, int n, const double *h_a,
                       const double *h_b, double *rel_rms, double *agreement);
/* fallen (may be NULL; one int per realization) receives 1 for the
 * realizations that fell back to the plain method. */
int fs_sg_ensemble_run(fs_batch *b, fs_surrogate *s, const fs_sg_ensemble_opts *o,
                       fs_sg_ensemble_stats *stats, int *fallen);

#ifdef __cplusplus
}
#endif

#endif /* FASTSCAPE_SURROGATE_H */
