// Device-side construction of very large fixed in-degree networks (sm_103a).
//
// The reference builds `connect(i='k for k in sample(N_pre, size=K)')` on the
// host with one mt19937 (templates/synapses_create_generator.cpp:85-153); at
// 1e9 synapses that loop takes hours.  Here every target neuron j draws its K
// distinct sources from a counter-based generator (Philox4x32-10, Salmon et al.,
// "Parallel random numbers: as easy as 1, 2, 3", SC'11), so targets are built in
// parallel and the network depends only on the seed.  The same procedure is
// restated on the CPU in oracle/scale_ref.c and the two agree bit for bit.
//
// Procedure for target j of pathway p (population of M sources, K <= 1024):
//   if K/M > 1/16: selection sampling over the M candidates, candidate c taken
//   when (M-c-1)*U53(ctr{c, j, p+1024, 255}) < K - selected;
//   otherwise round 0: candidate k = floor(u32(ctr{k, j, p, 0}) * M / 2^32)
//   sort; every candidate equal to its predecessor is redrawn with
//   ctr{k, j, p, r} (k its sorted position, r the round); repeat until unique.
//   delay of the synapse at sorted position k: dmin + dspan * U53(ctr{k, j, p, 255})
//   with U53 the reference's 53-bit composition of two 32-bit words
//   (templates/objects.cpp:448-453), quantised (int)(delay/dt + 0.5)
//   (brian2/synapses/spikequeue.h:85-95).
// The CSR over (source, delay slot) is built by a counting sort; each segment is
// then ordered by target, which makes the result independent of atomic order.
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <cuda_runtime.h>

#include "b200_scale.h"  // the C ABI this file implements (include/)

namespace {

struct u4 { uint32_t x, y, z, w; };

__host__ __device__ inline void b200s_mulhilo(uint32_t a, uint32_t b, uint32_t& hi, uint32_t& lo) {
  const uint64_t p = (uint64_t)a * (uint64_t)b;
  hi = (uint32_t)(p >> 32);
  lo = (uint32_t)p;
}

// Philox4x32 with 10 rounds: multipliers 0xD2511F53 / 0xCD9E8D57, key
// increments 0x9E3779B9 / 0xBB67AE85 (the published constants of the method).
__host__ __device__ inline u4 b200s_philox(u4 c, uint32_t k0, uint32_t k1) {
  for (int r = 0; r < 10; ++r) {
    uint32_t hi0, lo0, hi1, lo1;
    b200s_mulhilo(0xD2511F53u, c.x, hi0, lo0);
    b200s_mulhilo(0xCD9E8D57u, c.z, hi1, lo1);
    c = u4{hi1 ^ c.y ^ k0, lo1, hi0 ^ c.w ^ k1, lo0};
    k0 += 0x9E3779B9u;
    k1 += 0xBB67AE85u;
  }
  return c;
}

__host__ __device__ inline uint32_t b200s_draw(uint32_t k, uint32_t j, uint32_t p, uint32_t r,
                                               uint64_t seed, uint32_t M) {
  const u4 o = b200s_philox(u4{k, j, p, r}, (uint32_t)seed, (uint32_t)(seed >> 32));
  return (uint32_t)(((uint64_t)o.x * (uint64_t)M) >> 32);
}

__host__ __device__ inline double b200s_u53(uint32_t k, uint32_t j, uint32_t p, uint64_t seed) {
  const u4 o = b200s_philox(u4{k, j, p, 255u}, (uint32_t)seed, (uint32_t)(seed >> 32));
  const long a = (long)(o.x >> 5), b = (long)(o.y >> 6);
  return (a * 67108864.0 + b) / 9007199254740992.0;
}

// One CTA per target: K distinct sorted sources and their delay slots.
__global__ void __launch_bounds__(256) b200s_sample_kernel(uint64_t seed, uint32_t p, uint32_t M, int K,
                                                           int n_post, double dmin, double dspan, double dt,
                                                           int32_t* __restrict__ pre, uint8_t* __restrict__ slot,
                                                           int* __restrict__ err) {
  __shared__ uint32_t v[1024];
  __shared__ int s_dup;
  const int j = blockIdx.x;
  if (j >= n_post) return;
  if ((int64_t)K * 16 > (int64_t)M) {
    // dense: selection sampling over all M candidates (Knuth, TAOCP 2, 3.4.2,
    // algorithm S), in the form of templates/synapses_create_generator.cpp:131-137
    if (threadIdx.x == 0) {
      int sel = 0;
      for (uint32_t c = 0; c < M && sel < K; ++c) {
        const double U = b200s_u53(c, (uint32_t)j, p + 1024u, seed);
        if ((double)(M - (c + 1)) * U < (double)(K - sel)) v[sel++] = c;
      }
    }
    __syncthreads();
  } else {
  int P2 = 1;
  while (P2 < K) P2 <<= 1;
  for (int k = threadIdx.x; k < P2; k += blockDim.x)
    v[k] = k < K ? b200s_draw((uint32_t)k, (uint32_t)j, p, 0u, seed, M) : 0xFFFFFFFFu;
  __syncthreads();
  for (int round = 1; round <= 64; ++round) {
    // bitonic sort of P2 values
    for (int size = 2; size <= P2; size <<= 1) {
      for (int stride = size >> 1; stride > 0; stride >>= 1) {
        for (int t = threadIdx.x; t < P2 / 2; t += blockDim.x) {
          const int lo = 2 * t - (t & (stride - 1));
          const int hi = lo + stride;
          const bool up = (lo & size) == 0;
          const uint32_t a = v[lo], b = v[hi];
          if ((a > b) == up) { v[lo] = b; v[hi] = a; }
        }
        __syncthreads();
      }
    }
    if (threadIdx.x == 0) s_dup = 0;
    __syncthreads();
    // redraw every value equal to its predecessor (decided before any write)
    bool dup[4] = {false, false, false, false};
    int q = 0;
    for (int k = threadIdx.x; k < K; k += blockDim.x, ++q)
      if (q < 4) dup[q] = (k > 0 && v[k] == v[k - 1]);
    __syncthreads();
    q = 0;
    for (int k = threadIdx.x; k < K; k += blockDim.x, ++q)
      if (q < 4 && dup[q]) {
        v[k] = b200s_draw((uint32_t)k, (uint32_t)j, p, (uint32_t)round, seed, M);
        s_dup = 1;
      }
    __syncthreads();
    if (!s_dup) break;
    if (round == 64) {
      if (threadIdx.x == 0) atomicExch(err, 1);
      return;
    }
  }
  }
  for (int k = threadIdx.x; k < K; k += blockDim.x) {
    const size_t o = (size_t)j * K + k;
    pre[o] = (int32_t)v[k];
    const double d = dmin + dspan * b200s_u53((uint32_t)k, (uint32_t)j, p, seed);
    slot[o] = (uint8_t)(int)(d / dt + 0.5);
  }
}

__global__ void b200s_count_kernel(const int32_t* __restrict__ pre, const uint8_t* __restrict__ slot, int64_t n,
                                   int W, int dmin, int M, int* __restrict__ cnt, int* __restrict__ err) {
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < n; e += (int64_t)gridDim.x * blockDim.x) {
    const int32_t s = pre[e];
    const int d = (int)slot[e] - dmin;
    if (s < 0 || s >= M || d < 0 || d >= W) {  // never expected: record and skip
      atomicExch(err, 2);
      continue;
    }
    atomicAdd(&cnt[(int64_t)s * W + d], 1);
  }
}

// exclusive scan, int32 counts -> int64 offsets: per-block sums, serial scan of
// the block sums by one CTA, then per-block offsets
__global__ void b200s_scan_block(const int* __restrict__ in, int64_t n, int64_t* __restrict__ out,
                                 int64_t* __restrict__ bsum) {
  __shared__ int64_t s[1024];
  const int64_t base = (int64_t)blockIdx.x * 1024;
  const int t = threadIdx.x;
  const int64_t x = (base + t < n) ? in[base + t] : 0;
  s[t] = x;
  __syncthreads();
  for (int o = 1; o < 1024; o <<= 1) {
    const int64_t y = t >= o ? s[t - o] : 0;
    __syncthreads();
    s[t] += y;
    __syncthreads();
  }
  if (base + t < n) out[base + t] = s[t] - x;
  if (t == 1023) bsum[blockIdx.x] = s[t];
}

__global__ void b200s_scan_sums(int64_t* bsum, int64_t nb) {
  if (threadIdx.x != 0) return;
  int64_t acc = 0;
  for (int64_t b = 0; b < nb; ++b) {
    const int64_t x = bsum[b];
    bsum[b] = acc;
    acc += x;
  }
  bsum[nb] = acc;
}

__global__ void b200s_scan_add(int64_t* __restrict__ out, int64_t n, const int64_t* __restrict__ bsum) {
  const int64_t i = (int64_t)blockIdx.x * 1024 + threadIdx.x;
  if (i < n) out[i] += bsum[blockIdx.x];
}

__global__ void b200s_scatter_kernel(const int32_t* __restrict__ pre, const uint8_t* __restrict__ slot, int64_t n,
                                     int K, int W, int dmin, const int64_t* __restrict__ seg,
                                     int* __restrict__ fill, int32_t* __restrict__ post_csr) {
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < n; e += (int64_t)gridDim.x * blockDim.x) {
    const int64_t b = (int64_t)pre[e] * W + (slot[e] - dmin);
    const int64_t pos = seg[b] + atomicAdd(&fill[b], 1);
    post_csr[pos] = (int32_t)(e / K);
  }
}

// one warp per segment: sort targets ascending and write the source index
__global__ void b200s_sort_segments(const int64_t* __restrict__ seg, int64_t n_seg, int W, int src_off,
                                    int32_t* __restrict__ post_csr, int32_t* __restrict__ pre_csr) {
  const int lane = threadIdx.x & 31;
  const int64_t warp = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
  const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
  for (int64_t b = warp; b < n_seg; b += nwarps) {
    const int64_t lo = seg[b], hi = seg[b + 1];
    const int len = (int)(hi - lo);
    const int32_t src = (int32_t)(b / W) + src_off;
    for (int k = lane; k < len; k += 32) pre_csr[lo + k] = src;
    if (len <= 1) continue;
    if (len <= 32) {
      int32_t x = lane < len ? post_csr[lo + lane] : 0x7fffffff;
      for (int size = 2; size <= 32; size <<= 1)
        for (int stride = size >> 1; stride > 0; stride >>= 1) {
          const int32_t y = __shfl_xor_sync(0xffffffffu, x, stride);
          const bool lower = (lane & stride) == 0;
          const bool up = (lane & size) == 0;
          x = (lower == up) ? min(x, y) : max(x, y);
        }
      if (lane < len) post_csr[lo + lane] = x;
    } else if (lane == 0) {
      for (int a = 1; a < len; ++a) {  // insertion sort (segments this long are rare)
        const int32_t key = post_csr[lo + a];
        int c = a - 1;
        while (c >= 0 && post_csr[lo + c] > key) {
          post_csr[lo + c + 1] = post_csr[lo + c];
          --c;
        }
        post_csr[lo + c + 1] = key;
      }
    }
    __syncwarp();
  }
}

__global__ void b200s_outdeg_kernel(const int64_t* __restrict__ seg, int n_src, int W, int32_t* __restrict__ out) {
  for (int s = blockIdx.x * blockDim.x + threadIdx.x; s < n_src; s += gridDim.x * blockDim.x)
    out[s] = (int32_t)(seg[(int64_t)(s + 1) * W] - seg[(int64_t)s * W]);
}

template <typename T>
__global__ void b200s_fill_kernel(T* p, T v, int64_t n) {
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < n; e += (int64_t)gridDim.x * blockDim.x)
    p[e] = v;
}

thread_local char g_err[512];

int fail(const char* what, cudaError_t e) {
  snprintf(g_err, sizeof(g_err), "%s: %s", what, cudaGetErrorString(e));
  return 1;
}

}  // namespace

#define S_CU(call)                               \
  do {                                           \
    cudaError_t _e = (call);                     \
    if (_e != cudaSuccess) return fail(#call, _e); \
  } while (0)

extern "C" {

const char* b200s_last_error() { return g_err; }

// Builds the CSR over (source, delay slot) of one fixed in-degree pathway:
// n_post targets, each with K distinct sources from a population of n_src
// (stored with offset src_off, the population's first index in its group),
// delays dmin + dspan*U quantised with dt.  Device buffers are returned in
// *d_segptr (int64, n_src*(dmax-dmin+1)+1), *d_post, *d_pre (int32, n_post*K);
// free them with b200s_free.
int b200s_fixed_indegree_csr(uint64_t seed, int32_t path_id, int32_t n_src, int32_t src_off, int32_t n_post,
                             int32_t K, double dmin, double dspan, double dt, int32_t* slot_min,
                             int32_t* slot_max, int64_t** d_segptr, int32_t** d_post, int32_t** d_pre,
                             int64_t* n_syn) {
  g_err[0] = 0;
  if (K < 0 || K > 1024 || K > n_src || n_post < 0 || n_src <= 0) {
    snprintf(g_err, sizeof(g_err), "invalid sizes (K=%d, n_src=%d)", K, n_src);
    return B200S_STATUS_ARG;
  }
  const int s0 = (int)(dmin / dt + 0.5), s1 = (int)((dmin + dspan) / dt + 0.5);
  if (s0 < 0 || s1 > 255) {
    snprintf(g_err, sizeof(g_err), "delays out of the 0..255 step range");
    return B200S_STATUS_ARG;
  }
  const int W = s1 - s0 + 1;
  const int64_t n = (int64_t)n_post * K;
  int32_t* pre = nullptr;
  uint8_t* slot = nullptr;
  int *cnt = nullptr, *err = nullptr;
  int64_t *seg = nullptr, *bsum = nullptr;
  int32_t *post_csr = nullptr, *pre_csr = nullptr;
  const int64_t nb = (int64_t)n_src * W;
  S_CU(cudaMalloc(&pre, (size_t)n * 4 + 16));
  S_CU(cudaMalloc(&slot, (size_t)n + 16));
  S_CU(cudaMalloc(&err, 16));
  S_CU(cudaMemset(err, 0, 16));
  if (n_post > 0)
    b200s_sample_kernel<<<n_post, 256>>>(seed, (uint32_t)path_id, (uint32_t)n_src, K, n_post, dmin, dspan, dt,
                                         pre, slot, err);
  S_CU(cudaGetLastError());
  int h_err = 0;
  S_CU(cudaMemcpy(&h_err, err, 4, cudaMemcpyDeviceToHost));
  if (h_err) {  // a target did not get K distinct sources: stop before using them
    cudaFree(pre);
    cudaFree(slot);
    cudaFree(err);
    snprintf(g_err, sizeof(g_err), "sampling did not converge");
    return B200S_STATUS_NOT_CONVERGED;
  }
  S_CU(cudaMalloc(&cnt, (size_t)nb * 4 + 16));
  S_CU(cudaMemset(cnt, 0, (size_t)nb * 4 + 16));
  b200s_count_kernel<<<4096, 256>>>(pre, slot, n, W, s0, n_src, cnt, err);
  S_CU(cudaGetLastError());
  S_CU(cudaMemcpy(&h_err, err, 4, cudaMemcpyDeviceToHost));
  if (h_err) {
    cudaFree(pre); cudaFree(slot); cudaFree(err); cudaFree(cnt);
    snprintf(g_err, sizeof(g_err), "construction produced an out-of-range index");
    return B200S_STATUS_INDEX;
  }
  const int64_t nblk = (nb + 1023) / 1024;
  S_CU(cudaMalloc(&seg, (size_t)(nb + 1) * 8));
  S_CU(cudaMalloc(&bsum, (size_t)(nblk + 1) * 8));
  b200s_scan_block<<<(unsigned)nblk, 1024>>>(cnt, nb, seg, bsum);
  b200s_scan_sums<<<1, 32>>>(bsum, nblk);
  b200s_scan_add<<<(unsigned)nblk, 1024>>>(seg, nb, bsum);
  S_CU(cudaMemcpy(seg + nb, bsum + nblk, 8, cudaMemcpyDeviceToDevice));
  S_CU(cudaGetLastError());
  S_CU(cudaMemset(cnt, 0, (size_t)nb * 4 + 16));
  S_CU(cudaMalloc(&post_csr, (size_t)n * 4 + 16));
  S_CU(cudaMalloc(&pre_csr, (size_t)n * 4 + 16));
  b200s_scatter_kernel<<<4096, 256>>>(pre, slot, n, K, W, s0, seg, cnt, post_csr);
  S_CU(cudaGetLastError());
  b200s_sort_segments<<<4096, 256>>>(seg, nb, W, src_off, post_csr, pre_csr);
  S_CU(cudaGetLastError());
  S_CU(cudaMemcpy(&h_err, err, 4, cudaMemcpyDeviceToHost));
  cudaFree(pre);
  cudaFree(slot);
  cudaFree(cnt);
  cudaFree(err);
  cudaFree(bsum);
  if (h_err) {
    cudaFree(seg);
    cudaFree(post_csr);
    cudaFree(pre_csr);
    snprintf(g_err, sizeof(g_err), "sampling did not converge");
    return B200S_STATUS_NOT_CONVERGED;
  }
  *slot_min = s0;
  *slot_max = s1;
  *d_segptr = seg;
  *d_post = post_csr;
  *d_pre = pre_csr;
  *n_syn = n;
  return 0;
}

int b200s_free(void* p) {
  if (p) S_CU(cudaFree(p));
  return 0;
}

int b200s_fill_f32(float* p, float v, int64_t n) {
  b200s_fill_kernel<float><<<4096, 256>>>(p, v, n);
  S_CU(cudaGetLastError());
  S_CU(cudaDeviceSynchronize());
  return 0;
}

int b200s_fill_f64(double* p, double v, int64_t n) {
  b200s_fill_kernel<double><<<4096, 256>>>(p, v, n);
  S_CU(cudaGetLastError());
  S_CU(cudaDeviceSynchronize());
  return 0;
}

// Out-degree of every source of a CSR over (source, delay slot), to the host.
int b200s_outdegree(const int64_t* d_segptr, int32_t n_src, int32_t W, int32_t* host_out) {
  int32_t* d = nullptr;
  S_CU(cudaMalloc(&d, (size_t)n_src * 4 + 16));
  b200s_outdeg_kernel<<<1024, 256>>>(d_segptr, n_src, W, d);
  S_CU(cudaGetLastError());
  S_CU(cudaMemcpy(host_out, d, (size_t)n_src * 4, cudaMemcpyDeviceToHost));
  cudaFree(d);
  return 0;
}

int b200s_to_host(void* dst, const void* src, int64_t bytes) {
  S_CU(cudaMemcpy(dst, src, (size_t)bytes, cudaMemcpyDeviceToHost));
  return 0;
}

}  // extern "C"

// ---------------------------------------------------------------------------
// Allocation-free variant of b200s_fixed_indegree_csr.
//
// For callers that may not call cudaMalloc/cudaFree while they run: a host
// program whose device memory is owned by another framework's pool allocator
// (a cudaMalloc/cudaFree pair in the middle of its work would synchronise the
// whole device and bypass that pool), or a long-running loop with a fixed
// device-memory budget that rebuilds small networks between runs.  The caller
// passes the output buffers; the temporary arrays come from one fixed device
// array that every GPU loading this library holds until the process exits.
// ---------------------------------------------------------------------------
#define B200S_NOALLOC_SCRATCH_BYTES ((size_t)16 << 20)  // 16 MiB per device

static __device__ __align__(256) unsigned char b200s_noalloc_scratch[B200S_NOALLOC_SCRATCH_BYTES];

namespace {
std::mutex g_scratch_mu;
void* g_scratch_addr[256] = {nullptr};  // device address of the array, per device ordinal

// Device address of the scratch array on the current device.  Host code may
// not use the symbol itself (it names a host-side stand-in), so the address is
// looked up once per device with that device current, and cached.
int scratch_on_current_device(unsigned char** out) {
  int dev = 0;
  S_CU(cudaGetDevice(&dev));
  if (dev < 0 || dev >= 256) {
    snprintf(g_err, sizeof(g_err), "device ordinal %d out of range", dev);
    return B200S_STATUS_ARG;
  }
  std::lock_guard<std::mutex> lock(g_scratch_mu);
  if (!g_scratch_addr[dev]) {
    void* p = nullptr;
    S_CU(cudaGetSymbolAddress(&p, b200s_noalloc_scratch));
    g_scratch_addr[dev] = p;
  }
  *out = (unsigned char*)g_scratch_addr[dev];
  return 0;
}

size_t align256(size_t x) { return (x + 255) & ~(size_t)255; }
}  // namespace

extern "C" {

// Scratch bytes the allocation-free entry point needs for a pathway, or 0 if
// the sizes are invalid.  Larger requests are rejected by the entry point.
int64_t b200s_noalloc_scratch_bytes(int32_t n_src, int32_t n_post, int32_t K, double dmin, double dspan,
                                    double dt) {
  if (K < 0 || K > 1024 || K > n_src || n_post < 0 || n_src <= 0) return 0;
  const int s0 = (int)(dmin / dt + 0.5), s1 = (int)((dmin + dspan) / dt + 0.5);
  if (s0 < 0 || s1 > 255) return 0;
  const int64_t n = (int64_t)n_post * K, nb = (int64_t)n_src * (s1 - s0 + 1);
  const int64_t nblk = (nb + 1023) / 1024;
  return (int64_t)(align256((size_t)n * 4) + align256((size_t)n) + align256((size_t)nb * 4 + 16) +
                   align256((size_t)(nblk + 1) * 8) + 256);
}

// Same network as b200s_fixed_indegree_csr, written into caller-allocated
// device buffers: d_segptr with n_src*(slot_max-slot_min+1)+1 entries
// (cap_seg), d_post and d_pre with n_post*K entries (cap_syn).  Allocates
// nothing.  Its first call on a device looks up the scratch array's device
// address (and so loads this library onto that device); make that first call
// before any stream capture.  All calls share the one scratch array and leave
// their temporaries in it: calls that overlap on the GPU (several host threads,
// or several streams) race on it and must be serialised by the caller.  Runs on
// the legacy default stream and returns after the work has completed.
int b200s_fixed_indegree_csr_noalloc(uint64_t seed, int32_t path_id, int32_t n_src, int32_t src_off,
                                     int32_t n_post, int32_t K, double dmin, double dspan, double dt,
                                     int32_t* slot_min, int32_t* slot_max, int64_t* d_segptr, int64_t cap_seg,
                                     int32_t* d_post, int32_t* d_pre, int64_t cap_syn) {
  g_err[0] = 0;
  const int64_t need = b200s_noalloc_scratch_bytes(n_src, n_post, K, dmin, dspan, dt);
  if (need == 0) {
    snprintf(g_err, sizeof(g_err), "invalid sizes (K=%d, n_src=%d, n_post=%d) or delays", K, n_src, n_post);
    return B200S_STATUS_ARG;
  }
  if ((size_t)need > B200S_NOALLOC_SCRATCH_BYTES) {
    snprintf(g_err, sizeof(g_err),
             "network too large for the allocation-free path: needs %lld scratch bytes, the limit is %zu "
             "(use b200s_fixed_indegree_csr)", (long long)need, B200S_NOALLOC_SCRATCH_BYTES);
    return B200S_STATUS_SCRATCH_LIMIT;
  }
  const int s0 = (int)(dmin / dt + 0.5), s1 = (int)((dmin + dspan) / dt + 0.5);
  const int W = s1 - s0 + 1;
  const int64_t n = (int64_t)n_post * K, nb = (int64_t)n_src * W, nblk = (nb + 1023) / 1024;
  if (cap_seg < nb + 1 || cap_syn < n || !d_segptr || (n > 0 && (!d_post || !d_pre))) {
    snprintf(g_err, sizeof(g_err), "output buffers too small: need %lld segment and %lld synapse entries",
             (long long)(nb + 1), (long long)n);
    return B200S_STATUS_ARG;
  }
  unsigned char* base = nullptr;
  int r = scratch_on_current_device(&base);
  if (r) return r;
  int32_t* pre = (int32_t*)base;
  size_t off = align256((size_t)n * 4);
  uint8_t* slot = base + off;
  off += align256((size_t)n);
  int* cnt = (int*)(base + off);
  off += align256((size_t)nb * 4 + 16);
  int64_t* bsum = (int64_t*)(base + off);
  off += align256((size_t)(nblk + 1) * 8);
  int* err = (int*)(base + off);
  // the scratch keeps the previous call's contents: clear what must start at zero
  S_CU(cudaMemset(err, 0, 16));
  if (n_post > 0)
    b200s_sample_kernel<<<n_post, 256>>>(seed, (uint32_t)path_id, (uint32_t)n_src, K, n_post, dmin, dspan, dt,
                                         pre, slot, err);
  S_CU(cudaGetLastError());
  int h_err = 0;
  S_CU(cudaMemcpy(&h_err, err, 4, cudaMemcpyDeviceToHost));
  if (h_err) {
    snprintf(g_err, sizeof(g_err), "sampling did not converge");
    return B200S_STATUS_NOT_CONVERGED;
  }
  S_CU(cudaMemset(cnt, 0, (size_t)nb * 4 + 16));
  b200s_count_kernel<<<4096, 256>>>(pre, slot, n, W, s0, n_src, cnt, err);
  S_CU(cudaGetLastError());
  S_CU(cudaMemcpy(&h_err, err, 4, cudaMemcpyDeviceToHost));
  if (h_err) {
    snprintf(g_err, sizeof(g_err), "construction produced an out-of-range index");
    return B200S_STATUS_INDEX;
  }
  b200s_scan_block<<<(unsigned)nblk, 1024>>>(cnt, nb, d_segptr, bsum);
  b200s_scan_sums<<<1, 32>>>(bsum, nblk);
  b200s_scan_add<<<(unsigned)nblk, 1024>>>(d_segptr, nb, bsum);
  S_CU(cudaMemcpy(d_segptr + nb, bsum + nblk, 8, cudaMemcpyDeviceToDevice));
  S_CU(cudaGetLastError());
  S_CU(cudaMemset(cnt, 0, (size_t)nb * 4 + 16));
  b200s_scatter_kernel<<<4096, 256>>>(pre, slot, n, K, W, s0, d_segptr, cnt, d_post);
  S_CU(cudaGetLastError());
  b200s_sort_segments<<<4096, 256>>>(d_segptr, nb, W, src_off, d_post, d_pre);
  S_CU(cudaGetLastError());
  S_CU(cudaStreamSynchronize(0));  // the legacy default stream, which every launch above used
  *slot_min = s0;
  *slot_max = s1;
  return 0;
}

}  // extern "C"

extern "C" {

// Host evaluation of one draw, for tests of the generator itself.
uint32_t b200s_host_draw(uint32_t k, uint32_t j, uint32_t p, uint32_t r, uint64_t seed, uint32_t M) {
  return b200s_draw(k, j, p, r, seed, M);
}

}  // extern "C"
