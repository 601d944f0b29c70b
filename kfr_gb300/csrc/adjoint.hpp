// Adjoints (vector-Jacobian products) of the transforms, for gradient-based callers.  No counterpart in the
// reference, which has no differentiation; they are built from the same kernels plus small elementwise
// kernels.
//
// Convention for complex values (the one complex autograd uses): for a real loss L, the gradient carried by a
// complex array z is dL/dRe(z) + i dL/dIm(z).  With it, the gradient of the input of a linear map y = A x is
// A^H applied to the gradient of y, and for a map from real to complex values it is the real part of that.
//   complex DFT (unscaled):     forward^H = unscaled inverse, inverse^H = forward;
//   real DFT r2c (CCs / Perm):  grad_x = c2r(g with bins 1 .. N/2-1 halved)       (DC and Nyquist as they are);
//   real DFT c2r:               grad_Y = r2c(grad_x) with bins 1 .. N/2-1 doubled;
//   DCT-II (forward):           grad_x = DCT-III of g with the X0 term at full weight
//                               (the reference's inverse halves it, so g[0] is doubled first);
//   DCT-III (the inverse):      grad_x = DCT-II of g, then element 0 halved;
//   causal FIR y[t] = sum_m h[m] x[t-m] (convolve_filter from a reset state):
//                               grad_x[t] = sum_m h[m] g[t+m]            (the filter run backwards in time),
//                               grad_h[m] = sum_channels sum_t g[t] x[t-m] (a cross-correlation, m < M).
#pragma once

#include "plan.hpp"

namespace kfr_gpu
{

// out[s][k] = w_k * in[s][k] for `batch` spectra of `bins` values (c+1 for CCs, c for Perm, c = N/2): w = 1 at
// bin 0 and (CCs) bin c, `interior` elsewhere.  in may equal out.
template <typename T>
cudaError_t launch_spectrum_weight(void* out, const void* in, long long batch, long long bins, bool ccs, T interior,
                                   cudaStream_t st);
// out[s][e] = in[s][e], times f at e = 0 (real arrays of n values).  in may equal out.
template <typename T>
cudaError_t launch_scale_first(T* out, const T* in, long long batch, long long n, T f, cudaStream_t st);
// out[c][t] = in[c][n-1-t] for `channels` arrays of n reals.  out must not alias in.
template <typename T>
cudaError_t launch_reverse(T* out, const T* in, long long channels, long long n, cudaStream_t st);
// out[c][t] = t < n ? in[c][t] : 0 for channels arrays of `size` reals (in: n reals per channel).
template <typename T>
cudaError_t launch_pad(T* out, const T* in, long long channels, long long n, long long size, cudaStream_t st);
// acc[k] (+)= sum_c a[c][k] * conj(b[c][k]) over `channels` spectra of `bins` values; first: overwrite acc.
template <typename T>
cudaError_t launch_cmac_conj(void* acc, const void* a, const void* b, long long channels, long long bins, bool first,
                             cudaStream_t st);

// Gradients of the causal FIR filter y = h * x over `channels` signals of n samples (zero initial state).
// All pointers are device pointers; grad_x and grad_h may each be NULL (not wanted).  Synchronous on st.
template <typename T>
void fir_backward(const T* taps, long long ntaps, long long channels, long long n, const T* x, const T* grad_y,
                  T* grad_x, T* grad_h, cudaStream_t st);

} // namespace kfr_gpu
