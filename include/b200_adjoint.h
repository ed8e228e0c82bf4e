/*
 * b200_adjoint.h -- forward pass and adjoint (reverse-time) gradients of an
 * exact-linear LIF network (libb200_adjoint, brian2_gb300/csrc/b200_adjoint.cu).
 *
 * No counterpart in the reference: Brian2 has no gradient code.  The forward
 * pass restates, for one fixed model, what the reference's step loop does for
 * a CUBA-style NeuronGroup driven through on_pre synapses: exact linear update
 * (templates/stateupdate.cpp), threshold (templates/threshold.cpp), reset
 * (templates/reset.cpp) and on_pre accumulation (templates/synapses.cpp), all
 * under brian2/devices/cpp_standalone/.  The readout receives each hidden spike
 * at its linearly interpolated crossing time inside the step (the event term
 * the adjoint differentiates), so the spike rule is not smoothed.
 *
 * Model: I' = -I/taus (+W row per input spike), v' = (El - v + I)/taum;
 * v > Vt -> v = Vr.  Readout: same dynamics without threshold, driven by the
 * hidden spikes through W_out.
 *
 * ip[5] = {steps, K, n_in, n_h, n_o}; fp[6] = {dt, El, Vt, Vr, taus, taum}.
 * state0 = [v(n_h), I(n_h), vo(n_o), Io(n_o)].  Input spikes: CSR by step,
 * in_ptr[steps+1], in_ids ascending within a step.  Layouts: W[n_in][n_h],
 * W_out[n_h][n_o], vo_trace/io_trace[steps][n_o] (state after each step).
 * All pointers are device pointers except ip and fp (host); stream is a
 * cudaStream_t or 0.  n_h <= 4096, n_o <= 64.  Returns 0, or non-zero with a
 * message in b200a_last_error().
 */
#ifndef B200_ADJOINT_H
#define B200_ADJOINT_H
#include <stdint.h>
#ifdef __cplusplus
extern "C" {
#endif
const char* b200a_last_error(void);

/* Forward pass.  ckpt (ceil(steps/K) * (2 n_h + 2 n_o) entries), spike_count
 * (n_h) and io_trace may be NULL; the backward pass needs ckpt, vo_trace and
 * io_trace. */
int b200a_forward_f32(const int32_t* ip, const double* fp, const float* W, const float* W_out,
                      const int32_t* in_ptr, const int32_t* in_ids, const float* state0, float* vo_trace,
                      int32_t* spike_count, float* ckpt, float* io_trace, void* stream);
int b200a_forward_f64(const int32_t* ip, const double* fp, const double* W, const double* W_out,
                      const int32_t* in_ptr, const int32_t* in_ids, const double* state0, double* vo_trace,
                      int32_t* spike_count, double* ckpt, double* io_trace, void* stream);

/* The forward pass with the readout driven at the step grid: each hidden
 * spike adds W_out to Io at the end of its step, as the reference's on_pre
 * delivery does (templates/synapses.cpp:20-49; the same network written as a
 * Brian script with a SpikeGeneratorGroup input computes it).  It pins the
 * forward pass to the reference; the loss is then piecewise constant in the
 * spike times, so the adjoint pass differentiates the interpolated delivery
 * above instead.  Same arguments as b200a_forward_*. */
int b200a_forward_grid_f32(const int32_t* ip, const double* fp, const float* W, const float* W_out,
                           const int32_t* in_ptr, const int32_t* in_ids, const float* state0, float* vo_trace,
                           int32_t* spike_count, float* ckpt, float* io_trace, void* stream);
int b200a_forward_grid_f64(const int32_t* ip, const double* fp, const double* W, const double* W_out,
                           const int32_t* in_ptr, const int32_t* in_ids, const double* state0, double* vo_trace,
                           int32_t* spike_count, double* ckpt, double* io_trace, void* stream);

/* Adjoint pass: grad_vo[steps][n_o] = dL/dvo_trace.  Accumulates dL/dW into dW
 * and dL/dW_out into dW_out (zero them first); writes dL/dtaum to *dtaum.
 * segbuf: K * (2 n_h + 2 n_o) entries of scratch (the recomputed segment). */
int b200a_backward_f32(const int32_t* ip, const double* fp, const float* W, const float* W_out,
                       const int32_t* in_ptr, const int32_t* in_ids, const float* ckpt, const float* grad_vo,
                       float* segbuf, float* dW, float* dW_out, float* dtaum, const float* vo_trace,
                       const float* io_trace, const float* state0, void* stream);
int b200a_backward_f64(const int32_t* ip, const double* fp, const double* W, const double* W_out,
                       const int32_t* in_ptr, const int32_t* in_ids, const double* ckpt, const double* grad_vo,
                       double* segbuf, double* dW, double* dW_out, double* dtaum, const double* vo_trace,
                       const double* io_trace, const double* state0, void* stream);
#ifdef __cplusplus
}
#endif
#endif
