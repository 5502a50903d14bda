/*
 * fwant_surrogate — kernels of the learned waveform surrogate (no counterpart in the
 * reference, which always runs the full finite-difference solve).
 *
 * A small 3-D convolutional network maps a perturbation of the reference model (plus
 * features of the reference wavefield) to receiver waveforms, so that line-search
 * candidates can be screened without a solve; the solver (fwant_gb300.h) is its fallback
 * and the judge of its error.  These entry points are the network's forward, backward and
 * optimiser steps; the training loop and the data layout live in fwant_gb300/surrogate.py.
 *
 * Conventions
 *  - Every pointer is a device pointer on the current device; `stream` is a cudaStream_t
 *    (NULL = the default stream).  Calls are asynchronous and return a cudaError_t value
 *    (0 = launched).
 *  - Activations, gradients and accumulation are FP32; weights are read as BF16 (uint16_t
 *    bit patterns) and kept as FP32 master copies by the optimiser.
 *  - Volumes are NCDHW (batch, channel, depth, height, width); convolution weights are
 *    [Cout][Cin][3][3][3]; dense weights [Out][In].
 *  - Every reduction has a fixed order: results repeat bit for bit.
 */
#ifndef FWANT_SURROGATE_H
#define FWANT_SURROGATE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Partial-sum slots fwant_nn_mse needs in `scratch`. */
#define FWANT_NN_MSE_BLOCKS 1024

/* y = conv3d(x, w) + bias: 3x3x3 kernel, zero padding 1, stride 1 or 2; output
 * (D-1)/stride+1 per axis.  bias may be NULL. */
int fwant_nn_conv3d_fwd(const float* x, const uint16_t* w, const float* bias, float* y, int B, int Cin, int D,
                        int H, int W, int Cout, int stride, void* stream);

/* Gradients of fwant_nn_conv3d_fwd given dy: dx (may be NULL), dw and db (may be NULL). */
int fwant_nn_conv3d_bwd(const float* x, const uint16_t* w, const float* dy, float* dx, float* dw, float* db, int B,
                        int Cin, int D, int H, int W, int Cout, int stride, void* stream);

/* y[b][o] = sum_i x[b][i] w[o][i] + bias[o] (bias may be NULL). */
int fwant_nn_linear_fwd(const float* x, const uint16_t* w, const float* bias, float* y, int B, int In, int Out,
                        void* stream);

/* Gradients of fwant_nn_linear_fwd: dx (may be NULL), dw, db (may be NULL). */
int fwant_nn_linear_bwd(const float* x, const uint16_t* w, const float* dy, float* dx, float* dw, float* db, int B,
                        int In, int Out, void* stream);

/* Leaky ReLU in place, and its backward (dy *= slope where the output y is not > 0). */
int fwant_nn_lrelu_fwd(float* y, long long n, float slope, void* stream);
int fwant_nn_lrelu_bwd(const float* y, float* dy, long long n, float slope, void* stream);

/* loss = mean((y - t)^2) into *loss; dy = 2 (y - t) / n (dy may be NULL).  scratch holds
 * FWANT_NN_MSE_BLOCKS floats. */
int fwant_nn_mse(const float* y, const float* t, float* dy, float* loss, float* scratch, long long n, void* stream);

/* Adam step t (1-based) with decoupled weight decay wd on FP32 master weights w; writes
 * the BF16 copy w16 (may be NULL). */
int fwant_nn_adam(float* w, uint16_t* w16, const float* g, float* m, float* v, long long n, float lr, float b1,
                  float b2, float eps, float wd, int t, void* stream);

/* w16 = round-to-nearest-even BF16 of w. */
int fwant_nn_to_bf16(const float* w, uint16_t* w16, long long n, void* stream);

/* Fixed waveform basis: out[b][g][t] = sum_k coef[b][g][k] basis[g][k][t] (G groups of
 * K basis traces of T samples), and its backward dcoef[b][g][k] = sum_t dout basis. */
int fwant_nn_basis_fwd(const float* coef, const float* basis, float* out, int B, int G, int K, int T, void* stream);
int fwant_nn_basis_bwd(const float* dout, const float* basis, float* dcoef, int B, int G, int K, int T, void* stream);

/* y = a + s * b, elementwise. */
int fwant_nn_axpby(const float* a, const float* b, float s, float* y, long long n, void* stream);

#ifdef __cplusplus
}
#endif

#endif /* FWANT_SURROGATE_H */
