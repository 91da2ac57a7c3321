/*
 * bamf_cnn.h - the learned birth proposal: a small convolutional network that
 * maps a 16x16 ROI to a birth-position density over 4x4 sub-cells of every
 * pixel and to emitter-count logits 0..10, its synthetic training data, its
 * training on the GPU, and its inference into the sampler's LEARNED birth
 * tables (bamf_roi_batch.birth_cdf / birth_sub).
 *
 * No reference counterpart: the reference sampler proposes births from the
 * data residual (source/c/LibRJMCMC.cpp:1688-1736).  The network only shapes
 * a proposal; the sampler enters its exact density into the Hastings ratio,
 * so the posterior does not depend on it.
 *
 * Network (weights FP32 master copy, convolutions in BF16 with FP32
 * accumulation on the tensor cores, heads in FP32), spatial index
 * p = y + 16 x (the ROI pixel order), channels last:
 *   x0   = (sqrt(max(D, 0) + 3/8) - its ROI mean) / 4
 *   a1   = relu(conv3x3(x0; 1 -> 32))                  FP32
 *   a2-4 = relu(conv3x3(a_{l-1}; 32 -> 32))            BF16 x BF16 -> FP32
 *   loc  = conv1x1(a4; 32 -> 16): logit of sub-cell s = sy + 4 sx of pixel p;
 *          softmax over all 4096 (pixel, sub-cell) cells
 *   cnt  = linear(mean_p a4; 32 -> 11)
 * Parameter vector (FP32, BAMF_CNN_NPARAM values, in this order; conv
 * weights [out][in][kx][ky] with kx along x, the slow pixel axis):
 *   W1[32][1][3][3] b1[32] W2[32][32][3][3] b2[32] W3 b3 W4 b4
 *   Wl[16][32] bl[16] Wc[11][32] bc[11]
 * Loss of a ROI with n emitters at (x_e, y_e) inside it:
 *   -(1/n) sum_e log softmax(loc)[cell(x_e, y_e)]   (when n > 0)
 *   - log softmax(cnt)[min(n, 10)]
 * averaged over the batch.
 */
#ifndef BAMF_CNN_H
#define BAMF_CNN_H

#include <stdint.h>

#include "bamf.h"

#ifdef __cplusplus
extern "C" {
#endif

#define BAMF_CNN_SIDE 16
#define BAMF_CNN_CH 32
#define BAMF_CNN_COUNTS 11
#define BAMF_CNN_NPARAM 28955
#define BAMF_SYNTH_NMAX 16 /* emitters per generated ROI (more are clipped) */

/* Generator of 16x16 training / evaluation ROIs: the reference forward
 * model (source/c/LibRJMCMC.cpp:15-59: background plus per-emitter
 * erf-integrated Gaussian) with Poisson noise.  n ~ Poisson(mean_n) clipped
 * to BAMF_SYNTH_NMAX, positions uniform on [0, 16)^2, intensity
 * log-normal(ln i_median, i_logsd), background bg (uniform on [bg, bg_max]
 * when bg_max > bg), PSF sigma. */
typedef struct bamf_synth_params {
    float mean_n;
    float sigma;
    float i_median;
    float i_logsd;
    float bg;
    float bg_max;
} bamf_synth_params;

/* n ROIs numbered first .. first+n-1 of the stream `seed` (ROI k depends
 * only on (seed, k)), device pointers:
 *   data  [n][256] photon counts, y fastest
 *   n_em  [n] emitter count
 *   xyi   [n][BAMF_SYNTH_NMAX][3] X, Y, I of each emitter (zeros past n_em) */
bamf_status bamf_synth_generate(const bamf_synth_params *sp, uint32_t seed, uint64_t first, int n,
                                float *data, int32_t *n_em, float *xyi, void *stream);

typedef struct bamf_cnn bamf_cnn;

/* A network with He-initialised weights from `seed` (zero biases). */
bamf_status bamf_cnn_create(bamf_cnn **net, uint32_t seed);
void bamf_cnn_destroy(bamf_cnn *net);

/* FP32 parameter vector in the order above (host pointers). */
bamf_status bamf_cnn_get_params(bamf_cnn *net, float *params);
bamf_status bamf_cnn_set_params(bamf_cnn *net, const float *params);

/* Loss and parameter gradient of one batch of n ROIs (device inputs in the
 * layout of bamf_synth_generate, n <= 4096); loss and grad to host. */
bamf_status bamf_cnn_loss_grad(bamf_cnn *net, const float *data, const int32_t *n_em, const float *xyi,
                               int n, float *loss, float *grad);

/* `steps` Adam steps (beta 0.9 / 0.999, eps 1e-8, learning rate lr decayed
 * linearly to lr/10) on fresh generator batches of `batch` ROIs (ROIs
 * step*batch .. of stream data_seed), each step one CUDA-graph replay.
 * loss_trace (host, may be NULL) receives the batch loss of every step. */
bamf_status bamf_cnn_train(bamf_cnn *net, const bamf_synth_params *sp, int steps, int batch, float lr,
                           uint32_t data_seed, float *loss_trace);

/* `steps` Adam steps (as bamf_cnn_train, optimiser state from zero) on
 * caller-provided examples: n_examples device ROIs in the layout of
 * bamf_synth_generate (data [n][256], n_em [n], xyi [n][BAMF_SYNTH_NMAX][3];
 * counts above BAMF_SYNTH_NMAX are clipped), step i training on examples
 * i*batch .. i*batch+batch-1 modulo n_examples.  This is how the network
 * learns from states the sampler accepted (bamf_batch_results.pos_trace)
 * on data the generator does not describe. */
bamf_status bamf_cnn_train_examples(bamf_cnn *net, const float *data, const int32_t *n_em, const float *xyi,
                                    int n_examples, int steps, int batch, float lr, float *loss_trace);
/* Inference on n device ROIs of 16x16 (data [n][256]), into the sampler's
 * LEARNED tables for ROIs laid out back to back (ROI k at pixel 256 k):
 * cdf [n][256], sub [n][256][16], and count logits [n][11] (may be NULL). */
bamf_status bamf_cnn_infer(bamf_cnn *net, const float *data, int n, float *cdf, float *sub,
                           float *count_logits, void *stream);

/* Chain start states from the network's output (the count logits may only
 * initialise a chain; the target is unchanged): n0 = argmax of the count
 * logits (at most max_n <= BAMF_NMAX) emitters at the n0 most probable
 * sub-cell centres, taken greedily with cells within 1 px of a chosen one
 * suppressed, each with intensity `intensity`.  Writes the sampler's
 * bamf_roi_batch.init_n [n] and init_ixy [n][3][BAMF_NMAX] (device). */
bamf_status bamf_cnn_init_states(const float *cdf, const float *sub, const float *count_logits, int n,
                                 float intensity, int max_n, int32_t *init_n, float *init_ixy, void *stream);

#ifdef __cplusplus
}
#endif

#endif
