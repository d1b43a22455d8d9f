/*
 * spss_surrogate.h — learned surrogate of the stationary order parameters,
 * part of libspss_gpu.so.  No counterpart in the reference, which maps a phase
 * diagram only by simulating every parameter point (MPI_PARAMETER_SCAN in the
 * SimulationEngine*Ptr engines); here a small network, trained on the GPU on
 * results of batched simulations (spss_batch_*), predicts the time-averaged
 * order parameters of a point, and the simulation stays the judge of points
 * the network is unsure about.
 *
 * Network: 5 -> 128 -> 128 -> 128 -> 4, GELU (exact, erf form) after the three
 * hidden layers, linear output.  Weights and activations enter the matrix
 * products in BF16, products accumulate in FP32 (tcgen05 tensor-core MMA with
 * the accumulator in tensor memory); biases, pre-activations, the loss and the
 * optimiser state are FP32.  Inputs and targets are whatever features the
 * caller chooses (the Python layer standardises them).
 *
 * Parameters travel as one FP32 array of SPSS_MLP_PARAMS values, in this
 * order: W1[128][5], b1[128], W2[128][128], b2[128], W3[128][128], b3[128],
 * W4[4][128], b4[4] (W[out][in], y = W x + b).
 *
 * Every function returns SPSS_OK (0) or a negative SPSS_ERR_* code
 * (spss_gpu.h) and never aborts.  A handle is not thread-safe.
 */
#ifndef SPSS_SURROGATE_H
#define SPSS_SURROGATE_H

#include "spss_gpu.h"

#ifdef __cplusplus
extern "C" {
#endif

#define SPSS_MLP_INPUTS 5
#define SPSS_MLP_HIDDEN 128
#define SPSS_MLP_OUTPUTS 4
#define SPSS_MLP_PARAMS 34308

typedef struct spss_mlp spss_mlp;

/* A network with seeded initial weights (uniform in +-1/sqrt(fan_in), biases 0). */
int spss_mlp_create(unsigned long long seed, spss_mlp **out);
int spss_mlp_destroy(spss_mlp *m);
int spss_mlp_set_params(spss_mlp *m, const float *params, long len);
int spss_mlp_get_params(spss_mlp *m, float *params, long len);

/* y[n][4] = network(x[n][5]) for host arrays (n >= 1). */
int spss_mlp_forward(spss_mlp *m, const float *x, long n, float *y);

/* Loss and gradient of one batch of host arrays, parameters unchanged:
 * loss = (1/n) sum_i sum_o w[o] (y_io - t_io)^2, grad in the parameter order.
 * `w` holds 4 output weights (NULL: all 1). */
int spss_mlp_gradient(spss_mlp *m, const float *x, const float *t, const float *w, long n, float *grad, double *loss);

/* Training set resident on the GPU: x[n][5], t[n][4]. */
int spss_mlp_set_data(spss_mlp *m, const float *x, const float *t, long n);
/* Adam (beta1 0.9, beta2 0.999, eps 1e-8) on minibatches of `batch` rows
 * (a multiple of 128) of the resident set, `epochs` passes, each in an order
 * shuffled by a generator seeded with shuffle_seed + epoch; `w` as in
 * spss_mlp_gradient.  loss_per_epoch (NULL allowed) receives the mean
 * minibatch loss of every epoch. */
int spss_mlp_train(spss_mlp *m, int epochs, int batch, float lr, const float *w, unsigned long long shuffle_seed,
                   float *loss_per_epoch);
/* Number of tensor-core kernels this handle launched (forward, backward and
 * weight-gradient kernels). */
int spss_mlp_kernel_launches(spss_mlp *m, unsigned long long *count);

#ifdef __cplusplus
}
#endif

#endif
