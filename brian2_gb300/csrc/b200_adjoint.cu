// Exact-linear LIF network and its adjoint (sm_103a): gradients of a
// membrane-trace loss with respect to input weights W, readout weights W_out
// and the membrane time constant taum, without smoothing the spike rule.
//
// Network (per clock step n, t_n = n*dt; the hidden layer is the clock-driven
// CUBA LIF of the reference: exact propagation, threshold, reset on the grid):
//   vm   = El + a_m (v_n - El) + c I_n,   a_m = exp(-dt/taum), a_s = exp(-dt/taus),
//          c = taus (a_s - a_m) / (taus - taum)           (exact solution over dt)
//   spike if vm > Vt: crossing fraction phi = (Vt - v_n)/(vm - v_n), r = 1 - phi
//   v_{n+1} = spike ? Vr : vm;   I_{n+1} = a_s I_n + sum_j x_{n,j} W[j,:]
//   readout o (non-spiking, same dynamics) receives every hidden spike at its
//   interpolated time t_n + phi*dt:
//   vo_{n+1} = El + a_m (vo_n - El) + c Io_n + sum_h W_out[h,o] f(r_h)
//   Io_{n+1} = a_s Io_n + sum_h W_out[h,o] e(r_h),
//   e(r) = exp(-r dt/taus),  f(r) = taus (e(r) - exp(-r dt/taum)) / (taus - taum)
// Backward: the adjoint recursion of these equations in reverse time.  Event
// terms: at a hidden spike the adjoint of vm and v_n gets dL/dphi * dphi/d(.)
// (the crossing-time sensitivity) and nothing from v_{n+1} (the reset cuts it);
// each input spike adds lambda_I to dW; each hidden spike adds to dW_out.
// State is checkpointed every K steps in the forward pass; the backward pass
// recomputes each segment from its checkpoint.  One CTA runs the whole network
// (a clock step is a few thousand operations; the cost is latency).
//
// All buffers are caller-allocated device memory (plain pointers).
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cuda_runtime.h>

namespace {

template <typename T>
struct AdjP {
  int steps, K, n_in, n_h, n_o;
  T dt, El, Vt, Vr, taus, taum;
  // 1: the readout receives a hidden spike at the end of its step (the
  // reference's on_pre timing, templates/synapses.cpp) instead of at the
  // interpolated crossing time -- the forward pass only
  int grid;
};

template <typename T> __device__ __forceinline__ T ex(T x);
template <> __device__ __forceinline__ float ex<float>(float x) { return expf(x); }
template <> __device__ __forceinline__ double ex<double>(double x) { return exp(x); }

template <typename T>
struct Coef {
  T a_m, a_s, c;
  __device__ Coef(const AdjP<T>& P) {
    a_m = ex<T>(-P.dt / P.taum);
    a_s = ex<T>(-P.dt / P.taus);
    c = P.taus * (a_s - a_m) / (P.taus - P.taum);
  }
};

// f(r), e(r) and their derivatives in r and taum
template <typename T>
__device__ __forceinline__ void readout_kernel_fn(const AdjP<T>& P, T r, T& f, T& e, T& df_dr, T& de_dr,
                                                  T& df_dtaum) {
  const T es = ex<T>(-r * P.dt / P.taus), em = ex<T>(-r * P.dt / P.taum);
  const T d = P.taus - P.taum;
  e = es;
  f = P.taus * (es - em) / d;
  de_dr = -(P.dt / P.taus) * es;
  df_dr = P.taus * (-(P.dt / P.taus) * es + (P.dt / P.taum) * em) / d;
  const T dem_dtaum = em * r * P.dt / (P.taum * P.taum);
  df_dtaum = P.taus * (-dem_dtaum * d + (es - em)) / (d * d);
}

constexpr int MAXO = 64;
constexpr int MAXSPK = 4096;
constexpr int MAXIDS = 4096;  // input spikes of one segment staged in shared memory

// One clock step of the network held in shared memory; optional trace/raster.
template <typename T>
__device__ void step_forward(const AdjP<T>& P, const Coef<T>& C, int n, T* s_v, T* s_I, T* s_vo, T* s_Io,
                             int* s_spk, T* s_r, int* s_nspk, const T* __restrict__ W,
                             const T* __restrict__ Wout, const int* __restrict__ in_ptr,
                             const int* __restrict__ in_ids, T* vo_trace, int* spike_count,
                             T* io_trace = nullptr, bool readout = true) {
  // hidden neurons: update, threshold, crossing fraction, reset
  for (int h = threadIdx.x; h < P.n_h; h += blockDim.x) {
    const T v = s_v[h], I = s_I[h];
    const T vm = P.El + C.a_m * (v - P.El) + C.c * I;
    if (vm > P.Vt) {
      if (readout) {
        const int k = atomicAdd(s_nspk, 1);
        if (k < MAXSPK) {
          s_spk[k] = h;
          s_r[k] = P.grid ? (T)0 : (T)1 - (P.Vt - v) / (vm - v);  // (r = 0: f = 0, e = 1)
        }
      }
      s_v[h] = P.Vr;
      if (spike_count) spike_count[h] += 1;
    } else {
      s_v[h] = vm;
    }
    s_I[h] = C.a_s * I;
  }
  __syncthreads();
  // inputs of this step: I += W[j,:] in ascending j
  const int j0 = in_ptr[n], j1 = in_ptr[n + 1];
  for (int q = j0; q < j1; ++q) {
    const int j = in_ids[q];
    for (int h = threadIdx.x; h < P.n_h; h += blockDim.x) s_I[h] += W[(size_t)j * P.n_h + h];
  }
  // readout: spikes of this step in ascending neuron order (deterministic sums)
  const int ns = min(*s_nspk, MAXSPK);
  if (readout && threadIdx.x < P.n_o) {
    const int o = threadIdx.x;
    T av = 0, ai = 0;
    int last = -1;
    for (int c = 0; c < ns; ++c) {  // selection in ascending h without sorting the list
      int best = 0x7fffffff, bi = -1;
      for (int q = 0; q < ns; ++q)
        if (s_spk[q] > last && s_spk[q] < best) { best = s_spk[q]; bi = q; }
      last = best;
      T f, e, a, b, g;
      readout_kernel_fn(P, s_r[bi], f, e, a, b, g);
      const T w = Wout[(size_t)best * P.n_o + o];
      av += w * f;
      ai += w * e;
    }
    const T vo = s_vo[o], Io = s_Io[o];
    const T von = P.El + C.a_m * (vo - P.El) + C.c * Io + av;
    s_vo[o] = von;
    s_Io[o] = C.a_s * Io + ai;
    if (vo_trace) vo_trace[(size_t)n * P.n_o + o] = von;
    if (io_trace) io_trace[(size_t)n * P.n_o + o] = s_Io[o];
  }
  __syncthreads();
  if (readout) {
    if (threadIdx.x == 0) *s_nspk = 0;
    __syncthreads();
  }
}

// W_out in shared memory when it fits (every spike of every step reads a row)
template <typename T>
__device__ const T* stage_wout(const AdjP<T>& P, const T* Wout, T* s_wout, bool fits) {
  if (!fits) return Wout;
  for (int k = threadIdx.x; k < P.n_h * P.n_o; k += blockDim.x) s_wout[k] = Wout[k];
  return s_wout;
}

template <typename T>
__device__ void save_state(const AdjP<T>& P, T* dst, const T* s_v, const T* s_I, const T* s_vo, const T* s_Io) {
  for (int h = threadIdx.x; h < P.n_h; h += blockDim.x) {
    dst[h] = s_v[h];
    dst[P.n_h + h] = s_I[h];
  }
  if (threadIdx.x < P.n_o) {
    dst[2 * P.n_h + threadIdx.x] = s_vo[threadIdx.x];
    dst[2 * P.n_h + P.n_o + threadIdx.x] = s_Io[threadIdx.x];
  }
}

template <typename T>
__device__ void load_state(const AdjP<T>& P, const T* src, T* s_v, T* s_I, T* s_vo, T* s_Io) {
  for (int h = threadIdx.x; h < P.n_h; h += blockDim.x) {
    s_v[h] = src[h];
    s_I[h] = src[P.n_h + h];
  }
  if (threadIdx.x < P.n_o) {
    s_vo[threadIdx.x] = src[2 * P.n_h + threadIdx.x];
    s_Io[threadIdx.x] = src[2 * P.n_h + P.n_o + threadIdx.x];
  }
}

template <typename T>
__global__ void __launch_bounds__(1024, 1) forward_kernel(AdjP<T> P, const T* __restrict__ W,
                                                          const T* __restrict__ Wout,
                                                          const int* __restrict__ in_ptr,
                                                          const int* __restrict__ in_ids, const T* __restrict__ state0,
                                                          T* vo_trace, int* spike_count, T* ckpt, T* io_trace,
                                                          int wout_smem) {
  extern __shared__ __align__(16) unsigned char smem[];
  T* s_v = (T*)smem;
  T* s_I = s_v + P.n_h;
  T* s_vo = s_I + P.n_h;
  T* s_Io = s_vo + MAXO;
  T* s_r = s_Io + MAXO;
  int* s_spk = (int*)(s_r + MAXSPK);
  T* s_wout = (T*)(s_spk + MAXSPK);
  __shared__ int s_nspk;
  if (threadIdx.x == 0) s_nspk = 0;
  const Coef<T> C(P);
  load_state(P, state0, s_v, s_I, s_vo, s_Io);
  const T* Wo = stage_wout(P, Wout, s_wout, wout_smem != 0);
  __syncthreads();
  const int S = 2 * P.n_h + 2 * P.n_o;
  for (int n = 0; n < P.steps; ++n) {
    if (ckpt && n % P.K == 0) save_state(P, ckpt + (size_t)(n / P.K) * S, s_v, s_I, s_vo, s_Io);
    step_forward(P, C, n, s_v, s_I, s_vo, s_Io, s_spk, s_r, &s_nspk, W, Wo, in_ptr, in_ids, vo_trace, spike_count,
                 io_trace);
  }
}

template <typename T>
__device__ __forceinline__ T block_sum(T x, T* red) {
  for (int o = 16; o > 0; o >>= 1) x += __shfl_down_sync(0xffffffffu, x, o);
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  __syncthreads();
  if (lane == 0) red[w] = x;
  __syncthreads();
  T s = 0;
  if (threadIdx.x == 0)
    for (int k = 0; k < (int)(blockDim.x + 31) / 32; ++k) s += red[k];
  return s;  // valid in thread 0
}

// Reverse pass over all segments.  grad_vo[n*n_o+o] = dL/dvo_{n+1}.
template <typename T>
__global__ void __launch_bounds__(1024, 1) backward_kernel(AdjP<T> P, const T* __restrict__ W,
                                                           const T* __restrict__ Wout,
                                                           const int* __restrict__ in_ptr,
                                                           const int* __restrict__ in_ids,
                                                           const T* __restrict__ ckpt,
                                                           const T* __restrict__ grad_vo, T* segbuf, T* dW,
                                                           T* dWout, T* dtaum, const T* __restrict__ vo_trace,
                                                           const T* __restrict__ io_trace,
                                                           const T* __restrict__ state0, int wout_smem) {
  extern __shared__ __align__(16) unsigned char smem[];
  T* s_v = (T*)smem;
  T* s_I = s_v + P.n_h;
  T* s_vo = s_I + P.n_h;
  T* s_Io = s_vo + MAXO;
  T* s_r = s_Io + MAXO;
  int* s_spk = (int*)(s_r + MAXSPK);
  T* l_v = (T*)(s_spk + MAXSPK);
  T* l_I = l_v + P.n_h;
  __shared__ T l_vo[MAXO], l_Io[MAXO], s_Lvo[MAXO], s_lIo1[MAXO];
  __shared__ T red[32];
  __shared__ int s_nspk;
  if (threadIdx.x == 0) s_nspk = 0;
  const Coef<T> C(P);
  for (int h = threadIdx.x; h < P.n_h; h += blockDim.x) { l_v[h] = 0; l_I[h] = 0; }
  if (threadIdx.x < P.n_o) { l_vo[threadIdx.x] = 0; l_Io[threadIdx.x] = 0; }
  T p_am = 0, p_c = 0, p_ft = 0;  // per-thread partial sums for dL/dtaum
  const int S = 2 * P.n_h + 2 * P.n_o;
  const int nseg = (P.steps + P.K - 1) / P.K;
  __syncthreads();
  // per-segment staging in shared memory: dL/dvo rows, readout state, inputs
  T* s_g = l_I + P.n_h;                          // [K * n_o]
  T* s_ro = s_g + (size_t)P.K * P.n_o;           // [K * 2 n_o]: vo_n, Io_n
  int* s_ip = (int*)(s_ro + (size_t)P.K * 2 * P.n_o);  // [K + 1] input offsets
  int* s_ids = s_ip + P.K + 1;                   // [MAXIDS] input indices
  T* s_wout = (T*)(((uintptr_t)(s_ids + MAXIDS) + 15) & ~(uintptr_t)15);
  const T* Wo = stage_wout(P, Wout, s_wout, wout_smem != 0);
  const int h0 = threadIdx.x;
  const bool own = h0 < P.n_h;
  for (int seg = nseg - 1; seg >= 0; --seg) {
    const int s0 = seg * P.K, s1 = min(P.steps, s0 + P.K);
    // recompute the segment from its checkpoint, keeping the state at each step
    load_state(P, ckpt + (size_t)seg * S, s_v, s_I, s_vo, s_Io);
    __syncthreads();
    // the readout state of every step comes from the forward traces
    for (int k = threadIdx.x; k < (s1 - s0) * P.n_o; k += blockDim.x) {
      const int n = s0 + k / P.n_o, o = k % P.n_o;
      s_ro[(size_t)(n - s0) * 2 * P.n_o + o] =
          n == 0 ? state0[2 * P.n_h + o] : vo_trace[(size_t)(n - 1) * P.n_o + o];
      s_ro[(size_t)(n - s0) * 2 * P.n_o + P.n_o + o] =
          n == 0 ? state0[2 * P.n_h + P.n_o + o] : io_trace[(size_t)(n - 1) * P.n_o + o];
    }
    for (int n = s0; n < s1; ++n) {  // hidden layer only
      save_state(P, segbuf + (size_t)(n - s0) * S, s_v, s_I, s_vo, s_Io);
      step_forward(P, C, n, s_v, s_I, s_vo, s_Io, s_spk, s_r, &s_nspk, W, Wo, in_ptr, in_ids, (T*)nullptr,
                   (int*)nullptr, (T*)nullptr, false);
    }
    const int ib = in_ptr[s0], nin = in_ptr[s1] - ib;
    const bool ids_smem = nin <= MAXIDS;
    for (int k = threadIdx.x; k < (s1 - s0) * P.n_o; k += blockDim.x) s_g[k] = grad_vo[(size_t)s0 * P.n_o + k];
    for (int k = threadIdx.x; k <= s1 - s0; k += blockDim.x) s_ip[k] = in_ptr[s0 + k] - ib;
    if (ids_smem)
      for (int k = threadIdx.x; k < nin; k += blockDim.x) s_ids[k] = in_ids[ib + k];
    __syncthreads();
    // the state of step n is loaded one step ahead (its latency overlaps step n+1)
    T v_nx = 0, I_nx = 0;
    if (own) {
      v_nx = segbuf[(size_t)(s1 - 1 - s0) * S + h0];
      I_nx = segbuf[(size_t)(s1 - 1 - s0) * S + P.n_h + h0];
    }
    for (int n = s1 - 1; n >= s0; --n) {
      const int ln = n - s0;
      const T* st = segbuf + (size_t)ln * S;
      // readout adjoint: Lambda = lambda_vo(n+1) + dL/dvo(n+1)
      if (threadIdx.x < P.n_o) {
        const int o = threadIdx.x;
        const T L = l_vo[o] + s_g[(size_t)ln * P.n_o + o];
        s_Lvo[o] = L;
        s_lIo1[o] = l_Io[o];
        const T vo = s_ro[(size_t)ln * 2 * P.n_o + o], Io = s_ro[(size_t)ln * 2 * P.n_o + P.n_o + o];
        p_am += L * (vo - P.El);
        p_c += L * Io;
        l_vo[o] = C.a_m * L;
        l_Io[o] = C.c * L + C.a_s * l_Io[o];
      }
      __syncthreads();
      const int q0 = s_ip[ln], q1 = s_ip[ln + 1];
      for (int h = threadIdx.x; h < P.n_h; h += blockDim.x) {
        T v, I;
        if (h == h0) {
          v = v_nx;
          I = I_nx;
          if (n > s0) {
            v_nx = st[h0 - S];
            I_nx = st[P.n_h + h0 - S];
          }
        } else {
          v = st[h];
          I = st[P.n_h + h];
        }
        const T vm = P.El + C.a_m * (v - P.El) + C.c * I;
        const T lv1 = l_v[h], lI1 = l_I[h];
        // input weights: one reduction per input spike (this thread owns column h)
        for (int q = q0; q < q1; ++q) {
          const int j = ids_smem ? s_ids[q] : in_ids[ib + q];
          atomicAdd(&dW[(size_t)j * P.n_h + h], lI1);
        }
        T lvm, lv_dir = 0;
        if (vm > P.Vt) {
          const T dvm = vm - v;
          const T r = (T)1 - (P.Vt - v) / dvm;
          T f, e, df_dr, de_dr, df_dt;
          readout_kernel_fn(P, r, f, e, df_dr, de_dr, df_dt);
          T dLdr = 0;
          for (int o = 0; o < P.n_o; ++o) {
            const T w = Wo[(size_t)h * P.n_o + o];
            atomicAdd(&dWout[(size_t)h * P.n_o + o], s_Lvo[o] * f + s_lIo1[o] * e);
            dLdr += w * (s_Lvo[o] * df_dr + s_lIo1[o] * de_dr);
            p_ft += w * s_Lvo[o] * df_dt;
          }
          const T dLdphi = -dLdr;
          lvm = dLdphi * (-(P.Vt - v) / (dvm * dvm));  // dphi/dvm
          lv_dir = dLdphi * ((P.Vt - vm) / (dvm * dvm));  // dphi/dv_n
        } else {
          lvm = lv1;
        }
        l_v[h] = C.a_m * lvm + lv_dir;
        l_I[h] = C.c * lvm + C.a_s * lI1;
        p_am += lvm * (v - P.El);
        p_c += lvm * I;
      }
      __syncthreads();
    }
  }
  const T am = block_sum(p_am, red);
  const T cc = block_sum(p_c, red);
  const T ft = block_sum(p_ft, red);
  if (threadIdx.x == 0) {
    const T dam = C.a_m * P.dt / (P.taum * P.taum);
    const T d = P.taus - P.taum;
    const T dc = P.taus * (-dam * d + (C.a_s - C.a_m)) / (d * d);
    *dtaum = am * dam + cc * dc + ft;
  }
}

template <typename T>
size_t smem_bytes(const AdjP<T>& P, bool backward, bool wout) {
  size_t b = (size_t)(2 * P.n_h + 2 * MAXO + MAXSPK) * sizeof(T) + MAXSPK * sizeof(int);
  if (backward)
    b += (size_t)2 * P.n_h * sizeof(T) + (size_t)P.K * 3 * P.n_o * sizeof(T) + (size_t)(P.K + 1 + MAXIDS) * sizeof(int) + 16;
  if (wout) b += (size_t)P.n_h * P.n_o * sizeof(T) + 16;
  return b + 64;
}

constexpr size_t SMEM_LIMIT = 220 * 1024;

thread_local char g_err[256];

template <typename T>
int run_forward(const AdjP<T>& P, const T* W, const T* Wout, const int* in_ptr, const int* in_ids, const T* state0,
                T* vo_trace, int* spike_count, T* ckpt, T* io_trace, cudaStream_t s) {
  if (P.n_o > MAXO || P.n_h <= 0 || P.n_h > MAXSPK || P.steps < 0 || P.K <= 0) {
    snprintf(g_err, sizeof(g_err), "invalid sizes (n_h <= %d, n_o <= %d)", MAXSPK, MAXO);
    return 2;
  }
  const int wout = smem_bytes(P, false, true) <= SMEM_LIMIT ? 1 : 0;
  const size_t sm = smem_bytes(P, false, wout != 0);
  cudaError_t e = cudaFuncSetAttribute(forward_kernel<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
  if (e == cudaSuccess) {
    forward_kernel<T><<<1, 1024, sm, s>>>(P, W, Wout, in_ptr, in_ids, state0, vo_trace, spike_count, ckpt, io_trace,
                                          wout);
    e = cudaGetLastError();
  }
  if (e != cudaSuccess) {
    snprintf(g_err, sizeof(g_err), "forward launch: %s", cudaGetErrorString(e));
    return 1;
  }
  return 0;
}

template <typename T>
int run_backward(const AdjP<T>& P, const T* W, const T* Wout, const int* in_ptr, const int* in_ids, const T* ckpt,
                 const T* grad_vo, T* segbuf, T* dW, T* dWout, T* dtaum, const T* vo_trace, const T* io_trace,
                 const T* state0, cudaStream_t s) {
  if (P.n_o > MAXO || P.n_h <= 0 || P.n_h > MAXSPK || P.steps < 0 || P.K <= 0) {
    snprintf(g_err, sizeof(g_err), "invalid sizes (n_h <= %d, n_o <= %d)", MAXSPK, MAXO);
    return 2;
  }
  const int wout = smem_bytes(P, true, true) <= SMEM_LIMIT ? 1 : 0;
  const size_t sm = smem_bytes(P, true, wout != 0);
  if (sm > SMEM_LIMIT) {
    snprintf(g_err, sizeof(g_err), "network too large for one CTA (%zu bytes of shared memory)", sm);
    return 2;
  }
  cudaError_t e = cudaFuncSetAttribute(backward_kernel<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
  if (e == cudaSuccess) {
    backward_kernel<T><<<1, 1024, sm, s>>>(P, W, Wout, in_ptr, in_ids, ckpt, grad_vo, segbuf, dW, dWout, dtaum,
                                           vo_trace, io_trace, state0, wout);
    e = cudaGetLastError();
  }
  if (e != cudaSuccess) {
    snprintf(g_err, sizeof(g_err), "backward launch: %s", cudaGetErrorString(e));
    return 1;
  }
  return 0;
}

}  // namespace

extern "C" {

const char* b200a_last_error() { return g_err; }

// params: steps, K, n_in, n_h, n_o; dt, El, Vt, Vr, taus, taum.  state0 =
// [v(n_h), I(n_h), vo(n_o), Io(n_o)]; ckpt: ceil(steps/K)*(2 n_h + 2 n_o)
// entries or NULL; spike_count: n_h or NULL; stream: a cudaStream_t or 0.
int b200a_forward_f32(const int32_t* ip, const double* fp, const float* W, const float* Wout, const int32_t* in_ptr,
                      const int32_t* in_ids, const float* state0, float* vo_trace, int32_t* spike_count,
                      float* ckpt, float* io_trace, void* stream) {
  AdjP<float> P{ip[0], ip[1], ip[2], ip[3], ip[4], (float)fp[0], (float)fp[1], (float)fp[2], (float)fp[3],
                (float)fp[4], (float)fp[5]};
  return run_forward(P, W, Wout, in_ptr, in_ids, state0, vo_trace, spike_count, ckpt, io_trace,
                     (cudaStream_t)stream);
}
int b200a_forward_f64(const int32_t* ip, const double* fp, const double* W, const double* Wout, const int32_t* in_ptr,
                      const int32_t* in_ids, const double* state0, double* vo_trace, int32_t* spike_count,
                      double* ckpt, double* io_trace, void* stream) {
  AdjP<double> P{ip[0], ip[1], ip[2], ip[3], ip[4], fp[0], fp[1], fp[2], fp[3], fp[4], fp[5]};
  return run_forward(P, W, Wout, in_ptr, in_ids, state0, vo_trace, spike_count, ckpt, io_trace,
                     (cudaStream_t)stream);
}
// segbuf: K*(2 n_h + 2 n_o) entries; dW (n_in*n_h), dWout (n_h*n_o) are
// accumulated into (zero them first); dtaum: one entry, written; vo_trace and
// io_trace are the forward pass's traces, state0 its initial state.
// The forward pass with the readout driven at the step grid (each hidden spike
// adds W_out to Io at the end of its step, the reference's on_pre timing):
// the network as a Brian script with on_pre delivery computes it, so it pins
// the forward to the reference.  The loss is then piecewise constant in the
// spike times (no gradient through them), which is why the adjoint uses the
// interpolated delivery.
int b200a_forward_grid_f32(const int32_t* ip, const double* fp, const float* W, const float* Wout,
                           const int32_t* in_ptr, const int32_t* in_ids, const float* state0, float* vo_trace,
                           int32_t* spike_count, float* ckpt, float* io_trace, void* stream) {
  AdjP<float> P{ip[0], ip[1], ip[2], ip[3], ip[4], (float)fp[0], (float)fp[1], (float)fp[2], (float)fp[3],
                (float)fp[4], (float)fp[5], 1};
  return run_forward(P, W, Wout, in_ptr, in_ids, state0, vo_trace, spike_count, ckpt, io_trace,
                     (cudaStream_t)stream);
}
int b200a_forward_grid_f64(const int32_t* ip, const double* fp, const double* W, const double* Wout,
                           const int32_t* in_ptr, const int32_t* in_ids, const double* state0, double* vo_trace,
                           int32_t* spike_count, double* ckpt, double* io_trace, void* stream) {
  AdjP<double> P{ip[0], ip[1], ip[2], ip[3], ip[4], fp[0], fp[1], fp[2], fp[3], fp[4], fp[5], 1};
  return run_forward(P, W, Wout, in_ptr, in_ids, state0, vo_trace, spike_count, ckpt, io_trace,
                     (cudaStream_t)stream);
}
int b200a_backward_f32(const int32_t* ip, const double* fp, const float* W, const float* Wout, const int32_t* in_ptr,
                       const int32_t* in_ids, const float* ckpt, const float* grad_vo, float* segbuf, float* dW,
                       float* dWout, float* dtaum, const float* vo_trace, const float* io_trace, const float* state0,
                       void* stream) {
  AdjP<float> P{ip[0], ip[1], ip[2], ip[3], ip[4], (float)fp[0], (float)fp[1], (float)fp[2], (float)fp[3],
                (float)fp[4], (float)fp[5]};
  return run_backward(P, W, Wout, in_ptr, in_ids, ckpt, grad_vo, segbuf, dW, dWout, dtaum, vo_trace, io_trace, state0,
                      (cudaStream_t)stream);
}
int b200a_backward_f64(const int32_t* ip, const double* fp, const double* W, const double* Wout,
                       const int32_t* in_ptr, const int32_t* in_ids, const double* ckpt, const double* grad_vo,
                       double* segbuf, double* dW, double* dWout, double* dtaum, const double* vo_trace,
                       const double* io_trace, const double* state0, void* stream) {
  AdjP<double> P{ip[0], ip[1], ip[2], ip[3], ip[4], fp[0], fp[1], fp[2], fp[3], fp[4], fp[5]};
  return run_backward(P, W, Wout, in_ptr, in_ids, ckpt, grad_vo, segbuf, dW, dWout, dtaum, vo_trace, io_trace, state0,
                      (cudaStream_t)stream);
}

}  // extern "C"
