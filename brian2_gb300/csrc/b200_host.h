// Host runtime of the b200 step engine: the C ABI declared in include/b200.h.
//
// This file is included once by every generated model (.cu) after the model
// tables (b200_model_info) have been defined, so each model shared library is
// self-contained: one dlopen, one ctypes.CDLL.  It owns all device memory of a
// network ("handle"), builds the CSR/delay layout, tiles the neuron groups over
// CTAs, grows monitor buffers, launches the persistent step kernel and reports
// errors as status codes with a message (no exit() in library code).
#pragma once
#include <algorithm>
#include <cstdarg>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "b200_device.cuh"

#define B200_ERR_CUDA 1
#define B200_ERR_ARG 2
#define B200_ERR_CAPACITY 3
#define B200_STATUS_RANDOM_H 6  // B200_STATUS_RANDOM of include/b200.h

// ---------------------------------------------------------------------------
struct b200_dbuf {  // a device buffer owned by the handle
  void* p = nullptr;
  size_t bytes = 0;
};

struct b200_group_h {
  int32_t N = 0;
  std::vector<b200_dbuf> var;
  b200_dbuf gen_bins, gen_index, gen_last;  // spike generator lists and cursor
  int64_t gen_n = 0;
  int32_t gen_period = 0;
  std::vector<int32_t> tile_start, cta_tile;
  b200_dbuf d_tile_start, d_cta_tile, scratch, tile_cnt, ring, ring_total, ring_prefix;
  b200_dbuf S;
  int32_t R = 1;
  // push mode: each CTA's compact spike lists of the last RH steps, counts per slot and CTA
  b200_dbuf hist, hcnt;
  int32_t RH = 0, hist_ncta = 0;
};
struct b200_pathway_h {
  int32_t src_lo = 0, src_hi = 0, tgt_lo = 0, tgt_hi = 0;
  int32_t dmin = 0, dmax = 0;
  int64_t n_syn = 0;
  bool has_syn = false;
  std::vector<int64_t> perm;  // perm[csr position] = synapse index (creation order)
  b200_dbuf segptr, post, pre, S;
  b200_dbuf sidx;             // shared synapses: position of each entry in the owning pathway
  std::vector<b200_dbuf> var;
  // owner mode: synapses over (source, owning CTA), the payload variables in
  // that order, and the per-CTA event FIFOs
  b200_dbuf oseg, opost, odelay;
  std::vector<b200_dbuf> ovar;
  std::vector<int32_t> own_lo;  // ownership the layout was built for (empty: none)
  std::vector<int64_t> own_in;  // incoming synapses of each owning CTA
  bool own_stale = true;
  b200_dbuf ev_tgt, ev_state, ev_base, ev_tag, ev_off;
  std::vector<b200_dbuf> ev_pay;
  int64_t ev_cap = 0;
  int32_t ev_RB = 0, ev_W = 0, ev_ncta = 0;
};
struct b200_summed_h {
  int32_t lo = 0, hi = 0;
  b200_dbuf seg, syn;
};
struct b200_spkmon_h {
  int32_t lo = 0, hi = 0;
  int64_t cap = 0;
  b200_dbuf n, i, ts, count;
  b200_dbuf snap, vals;  // recorded variables: per-neuron values of the step, per-spike rows
  b200_dbuf xcnt;        // push mode: each CTA's recorded spikes of the last three steps
};
struct b200_ratemon_h {
  int32_t lo = 0, hi = 0;
  int64_t step0 = 0, cap = 0, n = 0;
  b200_dbuf cnt;
  b200_dbuf xcnt;        // push mode: each CTA's spikes of the last three steps
};
struct b200_statemon_h {
  int32_t n_rec = 0, n_vars = 0;
  std::vector<int32_t> idx, vars;
  int64_t step0 = 0, cap = 0;
  b200_dbuf d_idx, n, data;
};
struct b200_inst_h {
  std::vector<double> consts;
  std::vector<b200_group_h> g;
  std::vector<b200_pathway_h> p;
  std::vector<b200_spkmon_h> sm;
  std::vector<b200_ratemon_h> rm;
  std::vector<b200_statemon_h> stm;
  std::vector<b200_summed_h> sum;
  int32_t n_cta = 1;
  int64_t ts = 0;
  b200_dbuf bar, status, ts_done, pending, bar64;
  int32_t ran_owner = -1;  // mode of the runs so far with spikes in flight: -1 none, 0 classic, 1 owner, 2 push
  b200_dbuf acc[B200_MAX_ACC];  // push mode: deliveries not yet added, B200_PUSH_BUFS steps per variable
  // a launch failed part-way (timeout, index error, dropped events): the CTAs
  // stopped at different steps, so the state no longer belongs to one time
  // step; runs are refused until b200_set_step declares the step of the state
  bool stale = false;
  // random stream of the step loop: generator state on the device (624 words +
  // position; randn()'s kept value), and two buffers of draws; rng_buf[rng_cur]
  // holds the draws of steps [rng_from, rng_to), and the state is at rng_to
  b200_dbuf rng_state, rng_gauss, rng_buf[2];
  int rng_cur = 0;
  int64_t rng_from = 0, rng_to = 0;
  bool rng_set = false;
};

struct b200_net {
  const b200_model_info* M = nullptr;
  int n_inst = 0;
  double dt = 1e-4;
  std::vector<b200_inst_h> inst;
  b200_dbuf d_insts, d_cta_map, d_work;
  std::vector<b200_inst_d> h_insts;
  cudaStream_t stream = nullptr;
  int threads = 256;
  int min_blocks = 1;             // 2: register-capped variant, two CTAs per SM
  int max_tiles1 = 2, max_w = 1;  // dynamic shared-memory extents
  int state_bytes = 0;            // shared-memory state cache per CTA (0: none)
  bool smem_cache = true;         // cache the state of single-CTA instances
  bool profiling = false;         // per-phase clock64 profile of the step kernel
  bool use_clusters = true;       // instances of 2..16 CTAs run as thread-block clusters
  int allow_owner = 2;            // owner-mode delivery: 0 off, 1 on where possible, 2 auto
  int owner = 0;                  // 1: the current plan runs b200_owner_kernel
  int allow_push = 2;             // push-mode delivery: 0 off, 1 on where possible, 2 auto
  int push = 0;                   // 1: the current plan runs b200_push_kernel
  double ev_factor = 0.0;         // event FIFO records per CTA, in units of its incoming synapses (0: worst case)
  int cluster = 0;                // cluster size of the current launch plan (0: none)
  b200_dbuf prof;
  int queue_mode = 0;      // 1: single-CTA instances pulled from a work queue
  int grid = 0;
  int64_t chunk_steps = 100000;
  uint64_t limit_ns = 2000000000ull;  // bounded waits: 2 s
  int fault_rank = -1;                 // test hook: CTA that skips its first barrier
  bool prepared = false;
  bool use_graph = true;
  cudaGraphExec_t graph_exec = nullptr;
  int64_t graph_steps = -1;
  int64_t launches = 0;
  double last_run_ms = 0.0;
  double last_kernel_ms = 0.0;  // kernel launches only (CUDA events around them)
  std::string err;
  size_t device_bytes = 0;
  int tcode() const {
    return threads | ((min_blocks - 1) << 16) | (owner ? B200_TCODE_OWNER : 0) | (push ? B200_TCODE_PUSH : 0);
  }
  int mode() const { return push ? 2 : (owner ? 1 : 0); }
};

static int b200_fail(b200_net* n, int code, const char* fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof(buf), fmt, ap);
  va_end(ap);
  if (n) n->err = buf;
  return code;
}

#define B200_CU(net, call)                                                              \
  do {                                                                                  \
    cudaError_t _e = (call);                                                            \
    if (_e != cudaSuccess)                                                              \
      return b200_fail(net, B200_ERR_CUDA, "%s failed: %s (%s:%d)", #call,              \
                       cudaGetErrorString(_e), __FILE__, __LINE__);                     \
  } while (0)

static int b200_alloc(b200_net* n, b200_dbuf& b, size_t bytes, bool zero = true) {
  if (b.p && b.bytes >= bytes && bytes > 0) {
    if (zero) B200_CU(n, cudaMemsetAsync(b.p, 0, bytes, n->stream));
    return 0;
  }
  if (b.p) {
    cudaFree(b.p);
    n->device_bytes -= b.bytes;
    b.p = nullptr;
    b.bytes = 0;
  }
  size_t a = bytes ? bytes : 16;
  B200_CU(n, cudaMalloc(&b.p, a));
  b.bytes = a;
  n->device_bytes += a;
  if (zero) B200_CU(n, cudaMemsetAsync(b.p, 0, a, n->stream));
  return 0;
}
static void b200_free(b200_net* n, b200_dbuf& b) {
  if (b.p) {
    cudaFree(b.p);
    if (n) n->device_bytes -= b.bytes;
  }
  b.p = nullptr;
  b.bytes = 0;
}

extern "C" {

// ----------------------------------------------------------------- lifecycle
int b200_create(b200_net** out, int32_t n_inst, const int32_t* group_sizes, double dt) {
  if (!out || n_inst <= 0 || !group_sizes || !(dt > 0)) return B200_ERR_ARG;
  b200_net* n = new b200_net();
  n->M = &B200_MODEL;
  n->n_inst = n_inst;
  n->dt = dt;
  n->inst.resize(n_inst);
  cudaError_t e = cudaStreamCreateWithFlags(&n->stream, cudaStreamNonBlocking);
  if (e != cudaSuccess) {
    *out = n;
    return b200_fail(n, B200_ERR_CUDA, "cudaStreamCreate: %s", cudaGetErrorString(e));
  }
  const b200_model_info* M = n->M;
  for (int k = 0; k < n_inst; ++k) {
    b200_inst_h& I = n->inst[k];
    I.consts.assign(M->const_defaults, M->const_defaults + M->n_consts);
    I.g.resize(M->n_groups);
    I.p.resize(M->n_pathways);
    I.sm.resize(M->n_spkmon);
    I.rm.resize(M->n_ratemon);
    I.stm.resize(M->n_statemon);
    I.sum.resize(M->n_summed);
    for (int g = 0; g < M->n_groups; ++g) {
      b200_group_h& G = I.g[g];
      G.N = group_sizes[k * M->n_groups + g];
      if (G.N < 0) {
        *out = n;
        return b200_fail(n, B200_ERR_ARG, "negative group size");
      }
      G.var.resize(M->groups[g].n_vars);
      if (M->groups[g].alias >= 0) {  // a custom event's group: the state of the group it belongs to
        if (G.N != I.g[M->groups[g].alias].N) {
          *out = n;
          return b200_fail(n, B200_ERR_ARG, "group %d (events of group %d) has another size", g, M->groups[g].alias);
        }
        continue;
      }
      for (int v = 0; v < M->groups[g].n_vars; ++v) {
        // rounded up to 16 bytes: the update reads and writes whole groups of four neurons
        int r = b200_alloc(n, G.var[v], ((size_t)G.N * b200_kind_size(M->groups[g].var_kind[v]) + 15) & ~(size_t)15);
        if (r) {
          *out = n;
          return r;
        }
      }
    }
    for (int p = 0; p < M->n_pathways; ++p) {
      const b200_pathway_info& P = M->pathways[p];
      I.p[p].src_hi = I.g[P.src_group].N;
      I.p[p].tgt_hi = I.g[P.tgt_group].N;
      I.p[p].var.resize(P.n_vars);
    }
    for (int s = 0; s < M->n_spkmon; ++s) I.sm[s].hi = I.g[M->spkmon[s].group].N;
    for (int s = 0; s < M->n_ratemon; ++s) I.rm[s].hi = I.g[M->ratemon[s].group].N;
  }
  *out = n;
  return 0;
}

int b200_destroy(b200_net* n) {
  if (!n) return 0;
  cudaStreamSynchronize(n->stream);
  if (n->graph_exec) cudaGraphExecDestroy(n->graph_exec);
  for (auto& I : n->inst) {
    for (auto& G : I.g) {
      for (auto& b : G.var) b200_free(n, b);
      b200_free(n, G.gen_bins); b200_free(n, G.gen_index); b200_free(n, G.gen_last);
      b200_free(n, G.d_tile_start); b200_free(n, G.d_cta_tile); b200_free(n, G.scratch);
      b200_free(n, G.tile_cnt); b200_free(n, G.ring); b200_free(n, G.ring_total);
      b200_free(n, G.ring_prefix); b200_free(n, G.S);
      b200_free(n, G.hist); b200_free(n, G.hcnt);
    }
    for (auto& P : I.p) {
      for (auto& b : P.var) b200_free(n, b);
      b200_free(n, P.segptr); b200_free(n, P.post); b200_free(n, P.pre); b200_free(n, P.S); b200_free(n, P.sidx);
      for (auto& b : P.ovar) b200_free(n, b);
      for (auto& b : P.ev_pay) b200_free(n, b);
      b200_free(n, P.oseg); b200_free(n, P.opost); b200_free(n, P.odelay);
      b200_free(n, P.ev_tgt); b200_free(n, P.ev_state); b200_free(n, P.ev_base); b200_free(n, P.ev_tag);
      b200_free(n, P.ev_off);
    }
    for (auto& S : I.sm) {
      b200_free(n, S.n); b200_free(n, S.i); b200_free(n, S.ts); b200_free(n, S.count);
      b200_free(n, S.snap); b200_free(n, S.vals); b200_free(n, S.xcnt);
    }
    for (auto& S : I.rm) { b200_free(n, S.cnt); b200_free(n, S.xcnt); }
    for (auto& b : I.acc) b200_free(n, b);
    for (auto& S : I.stm) { b200_free(n, S.d_idx); b200_free(n, S.n); b200_free(n, S.data); }
    for (auto& S : I.sum) { b200_free(n, S.seg); b200_free(n, S.syn); }
    b200_free(n, I.rng_state); b200_free(n, I.rng_gauss); b200_free(n, I.rng_buf[0]); b200_free(n, I.rng_buf[1]);
    b200_free(n, I.bar); b200_free(n, I.status); b200_free(n, I.ts_done); b200_free(n, I.pending);
    b200_free(n, I.bar64);
  }
  b200_free(n, n->d_insts); b200_free(n, n->d_cta_map); b200_free(n, n->d_work); b200_free(n, n->prof);
  if (n->stream) cudaStreamDestroy(n->stream);
  delete n;
  return 0;
}

int b200_last_error(b200_net* n, char* buf, int64_t len) {
  if (!buf || len <= 0) return B200_ERR_ARG;
  const char* s = n ? n->err.c_str() : "null handle";
  snprintf(buf, (size_t)len, "%s", s);
  return 0;
}

// Launch shape.  threads: CTA size (32..1024, multiple of 32).  ctas_per_inst:
// CTAs cooperating on one instance (>1 uses the bounded instance barrier).
// queue_mode: 1 lets a grid of resident CTAs pull single-CTA instances from a
// work queue (batched sweeps).  chunk_steps: steps per kernel launch.
int b200_configure(b200_net* n, int32_t threads, const int32_t* ctas_per_inst, int32_t queue_mode,
                   int64_t chunk_steps, int32_t use_graph) {
  if (!n) return B200_ERR_ARG;
  if (threads < 32 || threads > B200_MAX_THREADS || threads % 32)
    return b200_fail(n, B200_ERR_ARG, "threads must be a multiple of 32 in [32,1024]");
  n->threads = threads;
  n->queue_mode = queue_mode ? 1 : 0;
  if (chunk_steps > 0) n->chunk_steps = chunk_steps;
  n->use_graph = use_graph != 0;
  for (int k = 0; k < n->n_inst; ++k) {
    int c = ctas_per_inst ? ctas_per_inst[k] : 1;
    if (c < 1) return b200_fail(n, B200_ERR_ARG, "ctas_per_inst must be >= 1");
    if (n->queue_mode && c != 1) return b200_fail(n, B200_ERR_ARG, "queue mode needs 1 CTA per instance");
    n->inst[k].n_cta = c;
  }
  n->prepared = false;
  return 0;
}

int b200_set_consts(b200_net* n, int32_t inst, const double* values, int32_t count) {
  if (!n || inst < 0 || inst >= n->n_inst || count != n->M->n_consts) return B200_ERR_ARG;
  n->inst[inst].consts.assign(values, values + count);
  n->prepared = false;
  return 0;
}

// kind 0: group state variable (obj = group, var = index); kind 1: synaptic
// variable (obj = pathway) given in synapse creation order.
static int b200_var_buf(b200_net* n, int32_t inst, int32_t kind, int32_t obj, int32_t var,
                        b200_dbuf** buf, int* vkind, int64_t* count) {
  if (!n || inst < 0 || inst >= n->n_inst) return b200_fail(n, B200_ERR_ARG, "bad instance");
  b200_inst_h& I = n->inst[inst];
  if (kind == 0) {
    if (obj < 0 || obj >= n->M->n_groups || var < 0 || var >= n->M->groups[obj].n_vars)
      return b200_fail(n, B200_ERR_ARG, "bad group variable %d/%d", obj, var);
    if (n->M->groups[obj].alias >= 0) obj = n->M->groups[obj].alias;  // a custom event's group: shared state
    *buf = &I.g[obj].var[var];
    *vkind = n->M->groups[obj].var_kind[var];
    *count = I.g[obj].N;
  } else if (kind == 1) {
    if (obj < 0 || obj >= n->M->n_pathways || var < 0 || var >= n->M->pathways[obj].n_vars)
      return b200_fail(n, B200_ERR_ARG, "bad synaptic variable %d/%d", obj, var);
    if (n->M->pathways[obj].alias >= 0) obj = n->M->pathways[obj].alias;  // shared synaptic variables
    if (!I.p[obj].has_syn) return b200_fail(n, B200_ERR_ARG, "synapses of pathway %d not set", obj);
    *buf = &I.p[obj].var[var];
    *vkind = n->M->pathways[obj].var_kind[var];
    *count = I.p[obj].n_syn;
  } else {
    return b200_fail(n, B200_ERR_ARG, "bad kind");
  }
  return 0;
}

int b200_upload(b200_net* n, int32_t inst, int32_t kind, int32_t obj, int32_t var,
                const void* src, int64_t count) {
  b200_dbuf* b;
  int vk;
  int64_t cnt;
  int r = b200_var_buf(n, inst, kind, obj, var, &b, &vk, &cnt);
  if (r) return r;
  if (kind == 1 && n->M->pathways[obj].alias >= 0) obj = n->M->pathways[obj].alias;
  if (count != cnt) return b200_fail(n, B200_ERR_ARG, "upload size %lld != %lld", (long long)count, (long long)cnt);
  const size_t es = b200_kind_size(vk);
  if (kind == 0) {
    B200_CU(n, cudaMemcpyAsync(b->p, src, (size_t)cnt * es, cudaMemcpyHostToDevice, n->stream));
  } else {
    // permute creation order -> CSR order
    const std::vector<int64_t>& perm = n->inst[inst].p[obj].perm;
    std::vector<char> tmp((size_t)cnt * es);
    const char* s = (const char*)src;
    for (int64_t k = 0; k < cnt; ++k) memcpy(&tmp[(size_t)k * es], s + (size_t)perm[k] * es, es);
    B200_CU(n, cudaMemcpyAsync(b->p, tmp.data(), tmp.size(), cudaMemcpyHostToDevice, n->stream));
    n->inst[inst].p[obj].own_stale = true;
    n->prepared = false;
  }
  B200_CU(n, cudaStreamSynchronize(n->stream));
  return 0;
}

int b200_download(b200_net* n, int32_t inst, int32_t kind, int32_t obj, int32_t var, void* dst,
                  int64_t count) {
  b200_dbuf* b;
  int vk;
  int64_t cnt;
  int r = b200_var_buf(n, inst, kind, obj, var, &b, &vk, &cnt);
  if (r) return r;
  if (kind == 1 && n->M->pathways[obj].alias >= 0) obj = n->M->pathways[obj].alias;
  if (count != cnt) return b200_fail(n, B200_ERR_ARG, "download size mismatch");
  const size_t es = b200_kind_size(vk);
  if (kind == 0) {
    B200_CU(n, cudaMemcpyAsync(dst, b->p, (size_t)cnt * es, cudaMemcpyDeviceToHost, n->stream));
    B200_CU(n, cudaStreamSynchronize(n->stream));
  } else {
    std::vector<char> tmp((size_t)cnt * es);
    B200_CU(n, cudaMemcpyAsync(tmp.data(), b->p, tmp.size(), cudaMemcpyDeviceToHost, n->stream));
    B200_CU(n, cudaStreamSynchronize(n->stream));
    const std::vector<int64_t>& perm = n->inst[inst].p[obj].perm;
    char* d = (char*)dst;
    for (int64_t k = 0; k < cnt; ++k) memcpy(d + (size_t)perm[k] * es, &tmp[(size_t)k * es], es);
  }
  return 0;
}

// Synapses of one pathway in creation order (brian2/synapses/synapses.py:2074):
// pre/post are indices within the source/target subgroup ranges
// [src_lo,src_hi) / [tgt_lo,tgt_hi) of their groups; delay_steps holds the
// quantised delay of each synapse, or NULL for the single delay `scalar_delay`.
// Replaces CSpikeQueue::prepare (brian2/synapses/spikequeue.h:45-105): the
// per-source synapse lists become one CSR over (source, delay slot), built by a
// stable counting sort so each segment keeps creation order.
int b200_set_synapses(b200_net* n, int32_t inst, int32_t pw, int32_t src_lo, int32_t src_hi,
                      int32_t tgt_lo, int32_t tgt_hi, const int32_t* pre, const int32_t* post,
                      const int32_t* delay_steps, int32_t scalar_delay, int64_t n_syn) {
  if (!n || inst < 0 || inst >= n->n_inst || pw < 0 || pw >= n->M->n_pathways)
    return b200_fail(n, B200_ERR_ARG, "bad instance/pathway");
  b200_inst_h& I = n->inst[inst];
  const b200_pathway_info& PI = n->M->pathways[pw];
  b200_pathway_h& P = I.p[pw];
  const int32_t Ns = I.g[PI.src_group].N, Nt = I.g[PI.tgt_group].N;
  if (src_lo < 0 || src_hi > Ns || src_lo > src_hi || tgt_lo < 0 || tgt_hi > Nt || tgt_lo > tgt_hi)
    return b200_fail(n, B200_ERR_ARG, "bad source/target range");
  if (n_syn < 0 || (n_syn > 0 && (!pre || !post))) return b200_fail(n, B200_ERR_ARG, "bad synapse arrays");
  const int32_t ns = src_hi - src_lo;
  int32_t dmin = 0, dmax = 0;
  if (delay_steps && n_syn > 0) {
    dmin = dmax = delay_steps[0];
    for (int64_t k = 0; k < n_syn; ++k) {
      dmin = std::min(dmin, delay_steps[k]);
      dmax = std::max(dmax, delay_steps[k]);
    }
    if (dmin < 0) return b200_fail(n, B200_ERR_ARG, "negative delay");
  } else {
    if (scalar_delay < 0) return b200_fail(n, B200_ERR_ARG, "negative delay");
    dmin = dmax = scalar_delay;
  }
  const int32_t W = dmax - dmin + 1;
  std::vector<int64_t> seg((size_t)ns * W + 1, 0);
  for (int64_t k = 0; k < n_syn; ++k) {
    const int32_t s = pre[k], t = post[k];
    if (s < 0 || s >= ns || t < 0 || t >= tgt_hi - tgt_lo)
      return b200_fail(n, B200_ERR_INDEX, "synapse %lld index out of range (pre %d, post %d)", (long long)k, s, t);
    const int32_t d = delay_steps ? delay_steps[k] - dmin : 0;
    seg[(size_t)s * W + d + 1]++;
  }
  for (size_t k = 1; k < seg.size(); ++k) seg[k] += seg[k - 1];
  std::vector<int64_t> fill(seg.begin(), seg.end() - 1);
  P.perm.assign((size_t)n_syn, 0);
  std::vector<int32_t> cpost((size_t)n_syn), cpre((size_t)n_syn);
  for (int64_t k = 0; k < n_syn; ++k) {
    const int32_t s = pre[k];
    const int32_t d = delay_steps ? delay_steps[k] - dmin : 0;
    const int64_t pos = fill[(size_t)s * W + d]++;
    P.perm[pos] = k;
    cpost[pos] = post[k] + tgt_lo;  // stored as index within the target group
    cpre[pos] = s + src_lo;         // index within the source group
  }
  int r;
  if (PI.alias >= 0) {
    // the on_post pathway of a Synapses object: the same synapses (creation
    // order) as its on_pre pathway, whose arrays hold the synaptic variables
    const b200_pathway_h& O = I.p[PI.alias];
    if (!O.has_syn || O.n_syn != n_syn)
      return b200_fail(n, B200_ERR_ARG, "pathway %s shares the synapses of %s: set those first (same synapses)",
                       PI.name, n->M->pathways[PI.alias].name);
    std::vector<int64_t> inv((size_t)n_syn), sx((size_t)n_syn);
    for (int64_t q = 0; q < n_syn; ++q) inv[(size_t)O.perm[q]] = q;
    for (int64_t q = 0; q < n_syn; ++q) sx[q] = inv[(size_t)P.perm[q]];
    if ((r = b200_alloc(n, P.sidx, (size_t)std::max<int64_t>(n_syn, 1) * 8, false))) return r;
    if (n_syn) B200_CU(n, cudaMemcpyAsync(P.sidx.p, sx.data(), (size_t)n_syn * 8, cudaMemcpyHostToDevice, n->stream));
  }
  P.src_lo = src_lo; P.src_hi = src_hi; P.tgt_lo = tgt_lo; P.tgt_hi = tgt_hi;
  P.dmin = dmin; P.dmax = dmax; P.n_syn = n_syn; P.has_syn = true;
  P.own_stale = true;
  if ((r = b200_alloc(n, P.segptr, seg.size() * 8, false))) return r;
  if ((r = b200_alloc(n, P.post, (size_t)n_syn * 4, false))) return r;
  if ((r = b200_alloc(n, P.pre, (size_t)n_syn * 4, false))) return r;
  B200_CU(n, cudaMemcpyAsync(P.segptr.p, seg.data(), seg.size() * 8, cudaMemcpyHostToDevice, n->stream));
  if (n_syn) {
    B200_CU(n, cudaMemcpyAsync(P.post.p, cpost.data(), (size_t)n_syn * 4, cudaMemcpyHostToDevice, n->stream));
    B200_CU(n, cudaMemcpyAsync(P.pre.p, cpre.data(), (size_t)n_syn * 4, cudaMemcpyHostToDevice, n->stream));
  }
  if (PI.alias < 0)
    for (int v = 0; v < PI.n_vars; ++v)
      if ((r = b200_alloc(n, P.var[v], (size_t)n_syn * b200_kind_size(PI.var_kind[v])))) return r;
  // summed variables over these synapses: per target neuron, its synapses'
  // positions in this pathway's order, in creation order (the order of the
  // reference's sum, templates/summed_variable.cpp:19-25)
  for (int sv = 0; sv < n->M->n_summed; ++sv) {
    const b200_summed_info& SI = n->M->summed[sv];
    if (SI.pathway != pw) continue;
    b200_summed_h& S = I.sum[sv];
    S.lo = SI.index_post ? tgt_lo : src_lo;
    S.hi = SI.index_post ? tgt_hi : src_hi;
    const int32_t nt = S.hi - S.lo;
    std::vector<int64_t> inv((size_t)n_syn), sseg((size_t)nt + 1, 0), ssyn((size_t)n_syn);
    for (int64_t q = 0; q < n_syn; ++q) inv[(size_t)P.perm[q]] = q;
    for (int64_t k = 0; k < n_syn; ++k) sseg[(size_t)(SI.index_post ? post[k] : pre[k]) + 1]++;
    for (size_t t = 1; t < sseg.size(); ++t) sseg[t] += sseg[t - 1];
    std::vector<int64_t> sfill(sseg.begin(), sseg.end() - 1);
    for (int64_t k = 0; k < n_syn; ++k) ssyn[(size_t)sfill[(size_t)(SI.index_post ? post[k] : pre[k])]++] = inv[k];
    if ((r = b200_alloc(n, S.seg, sseg.size() * 8, false))) return r;
    if ((r = b200_alloc(n, S.syn, (size_t)std::max<int64_t>(n_syn, 1) * 8, false))) return r;
    B200_CU(n, cudaMemcpyAsync(S.seg.p, sseg.data(), sseg.size() * 8, cudaMemcpyHostToDevice, n->stream));
    if (n_syn) B200_CU(n, cudaMemcpyAsync(S.syn.p, ssyn.data(), (size_t)n_syn * 8, cudaMemcpyHostToDevice, n->stream));
  }
  B200_CU(n, cudaStreamSynchronize(n->stream));
  n->prepared = false;
  return 0;
}

// Adopts a CSR that was built on the device (scale-mode construction).  The
// arrays are copied; the synapse order is the CSR order itself.
int b200_set_synapses_csr(b200_net* n, int32_t inst, int32_t pw, int32_t src_lo, int32_t src_hi,
                          int32_t tgt_lo, int32_t tgt_hi, int32_t dmin, int32_t dmax,
                          const int64_t* d_segptr, const int32_t* d_post, const int32_t* d_pre,
                          int64_t n_syn) {
  if (!n || inst < 0 || inst >= n->n_inst || pw < 0 || pw >= n->M->n_pathways)
    return b200_fail(n, B200_ERR_ARG, "bad instance/pathway");
  b200_inst_h& I = n->inst[inst];
  const b200_pathway_info& PI = n->M->pathways[pw];
  b200_pathway_h& P = I.p[pw];
  if (PI.alias >= 0) return b200_fail(n, B200_ERR_ARG, "pathway %s shares synapses: set them with b200_set_synapses", PI.name);
  if (dmin < 0 || dmax < dmin) return b200_fail(n, B200_ERR_ARG, "bad delay range");
  const int64_t nseg = (int64_t)(src_hi - src_lo) * (dmax - dmin + 1) + 1;
  int r;
  if ((r = b200_alloc(n, P.segptr, (size_t)nseg * 8, false))) return r;
  if ((r = b200_alloc(n, P.post, (size_t)n_syn * 4, false))) return r;
  if ((r = b200_alloc(n, P.pre, (size_t)n_syn * 4, false))) return r;
  B200_CU(n, cudaMemcpyAsync(P.segptr.p, d_segptr, (size_t)nseg * 8, cudaMemcpyDeviceToDevice, n->stream));
  B200_CU(n, cudaMemcpyAsync(P.post.p, d_post, (size_t)n_syn * 4, cudaMemcpyDeviceToDevice, n->stream));
  B200_CU(n, cudaMemcpyAsync(P.pre.p, d_pre, (size_t)n_syn * 4, cudaMemcpyDeviceToDevice, n->stream));
  P.perm.resize((size_t)n_syn);
  for (int64_t k = 0; k < n_syn; ++k) P.perm[k] = k;
  P.src_lo = src_lo; P.src_hi = src_hi; P.tgt_lo = tgt_lo; P.tgt_hi = tgt_hi;
  P.dmin = dmin; P.dmax = dmax; P.n_syn = n_syn; P.has_syn = true;
  P.own_stale = true;
  for (int v = 0; v < PI.n_vars; ++v)
    if ((r = b200_alloc(n, P.var[v], (size_t)n_syn * b200_kind_size(PI.var_kind[v])))) return r;
  B200_CU(n, cudaStreamSynchronize(n->stream));
  n->prepared = false;
  return 0;
}

// Device pointer of a synaptic variable (CSR order), for device-side fills.
int b200_synapse_var_ptr(b200_net* n, int32_t inst, int32_t pw, int32_t var, void** out) {
  b200_dbuf* b;
  int vk;
  int64_t cnt;
  int r = b200_var_buf(n, inst, 1, pw, var, &b, &vk, &cnt);
  if (r) return r;
  if (n->M->pathways[pw].alias >= 0) pw = n->M->pathways[pw].alias;
  *out = b->p;
  n->inst[inst].p[pw].own_stale = true;  // the caller may write it: owner copies are rebuilt
  n->prepared = false;
  return 0;
}

int b200_set_monitor_range(b200_net* n, int32_t inst, int32_t kind, int32_t mon, int32_t lo, int32_t hi) {
  if (!n || inst < 0 || inst >= n->n_inst) return B200_ERR_ARG;
  b200_inst_h& I = n->inst[inst];
  if (kind == 0 && mon >= 0 && mon < n->M->n_spkmon) {
    const int32_t N = I.g[n->M->spkmon[mon].group].N;
    if (lo < 0 || hi > N || lo > hi) return b200_fail(n, B200_ERR_ARG, "bad monitor range");
    I.sm[mon].lo = lo; I.sm[mon].hi = hi;
  } else if (kind == 1 && mon >= 0 && mon < n->M->n_ratemon) {
    const int32_t N = I.g[n->M->ratemon[mon].group].N;
    if (lo < 0 || hi > N || lo > hi) return b200_fail(n, B200_ERR_ARG, "bad monitor range");
    I.rm[mon].lo = lo; I.rm[mon].hi = hi;
  } else {
    return b200_fail(n, B200_ERR_ARG, "bad monitor");
  }
  n->prepared = false;
  return 0;
}

// StateMonitor: record variables `vars` of neurons `idx` at the start of every step.
int b200_set_statemon(b200_net* n, int32_t inst, int32_t mon, const int32_t* idx, int32_t n_rec,
                      const int32_t* vars, int32_t n_vars) {
  if (!n || inst < 0 || inst >= n->n_inst || mon < 0 || mon >= n->M->n_statemon) return B200_ERR_ARG;
  if (n_vars > 8 || n_vars < 0 || n_rec < 0) return b200_fail(n, B200_ERR_ARG, "bad state monitor");
  b200_statemon_h& S = n->inst[inst].stm[mon];
  const int g = n->M->statemon[mon].group, sp = n->M->statemon[mon].syn;
  // a neuron group's monitor: neuron indices; a Synapses object's: synapse indices (creation
  // order, checked against the synapses when the run is prepared)
  for (int k = 0; k < n_rec; ++k)
    if (idx[k] < 0 || (sp < 0 && idx[k] >= n->inst[inst].g[g].N))
      return b200_fail(n, B200_ERR_INDEX, "bad record index");
  const int nv = sp < 0 ? n->M->groups[g].n_vars : n->M->pathways[sp].n_vars;
  for (int k = 0; k < n_vars; ++k)
    if (vars[k] < 0 || vars[k] >= nv) return b200_fail(n, B200_ERR_ARG, "bad var");
  S.idx.assign(idx, idx + n_rec);
  S.vars.assign(vars, vars + n_vars);
  S.n_rec = n_rec;
  S.n_vars = n_vars;
  n->prepared = false;
  return 0;
}

}  // extern "C"

// ----------------------------------------------------------------- prepare
// Tiles of one group: contiguous neuron ranges, each owned by one CTA, whose
// boundaries include every source/monitor range boundary so that the spikes of
// any such range are a contiguous run of tiles.
static void b200_make_tiles(int32_t N, int n_cta, std::vector<int32_t> cuts,
                            std::vector<int32_t>& tile_start, std::vector<int32_t>& cta_tile) {
  cuts.push_back(0);
  cuts.push_back(N);
  // CTA ranges start at multiples of 4 neurons (16-byte aligned state accesses)
  const int32_t target = std::max<int32_t>(4, (((N + n_cta - 1) / n_cta) + 3) & ~3);
  for (int32_t x = target; x < N; x += target) cuts.push_back(x);
  std::sort(cuts.begin(), cuts.end());
  cuts.erase(std::unique(cuts.begin(), cuts.end()), cuts.end());
  tile_start = cuts;  // tiles [cuts[u], cuts[u+1])
  const int n_tiles = (int)tile_start.size() - 1;
  cta_tile.assign(n_cta + 1, n_tiles);
  // CTA c owns the tiles whose start lies in [c*target, (c+1)*target)
  int u = 0;
  for (int c = 0; c < n_cta; ++c) {
    cta_tile[c] = u;
    const int64_t end = (int64_t)(c + 1) * target;
    while (u < n_tiles && tile_start[u] < end) ++u;
  }
  cta_tile[n_cta] = n_tiles;
}

static int64_t b200_pow2ceil(int64_t x) {
  int64_t p = 1;
  while (p < x) p <<= 1;
  return p;
}

// Owner mode, one pathway of instance k: the synapses regrouped over (source,
// owning CTA) (rebuilt when the synapses or the ownership changed), the per-CTA
// event FIFOs, and the descriptor pointing at them.
static int b200_owner_pathway(b200_net* n, int k, int p, b200_pathway_d& PD) {
  const b200_model_info* M = n->M;
  b200_inst_h& I = n->inst[k];
  b200_pathway_h& P = I.p[p];
  const b200_pathway_info& PI = M->pathways[p];
  const b200_group_h& TG = I.g[PI.tgt_group];
  const int C = I.n_cta;
  std::vector<int32_t> own_lo(C + 1);
  for (int r = 0; r <= C; ++r) own_lo[r] = TG.tile_start[TG.cta_tile[r]];
  const bool delays = P.dmax >= 1 && P.n_syn > 0;
  if (!P.own_lo.empty() && P.own_lo != own_lo && I.ts > 0 && delays)
    return b200_fail(n, B200_ERR_ARG,
                     "pathway %s: the CTA count of a network with delays cannot change once it has run in "
                     "owner mode (events in flight belong to their CTA)", PI.name);
  int r;
  const int64_t n_src = P.src_hi - P.src_lo;
  if (P.own_stale || P.own_lo != own_lo) {
    if ((r = b200_alloc(n, P.oseg, (size_t)(n_src * C + 1) * 8, false))) return r;
    if ((r = b200_alloc(n, P.opost, (size_t)std::max<int64_t>(P.n_syn, 1) * 4, false))) return r;
    if ((r = b200_alloc(n, P.odelay, (size_t)std::max<int64_t>(P.n_syn, 1) * 2, false))) return r;
    P.ovar.resize(PI.n_payload);
    b200_relayout_args A;
    memset(&A, 0, sizeof(A));
    A.segptr = (const int64_t*)P.segptr.p;
    A.post = (const int32_t*)P.post.p;
    A.n_var = PI.n_payload;
    for (int m = 0; m < PI.n_payload; ++m) {
      const int v = PI.payload_var[m];
      const size_t es = b200_kind_size(PI.var_kind[v]);
      if (es != 4 && es != 8) return b200_fail(n, B200_ERR_ARG, "owner mode: unsupported synaptic variable size");
      if ((r = b200_alloc(n, P.ovar[m], (size_t)std::max<int64_t>(P.n_syn, 1) * es, false))) return r;
      A.var[m] = P.var[v].p;
      A.var_size[m] = (int32_t)es;
      A.ovar[m] = P.ovar[m].p;
    }
    A.n_src = (int32_t)n_src;
    A.W = P.dmax - P.dmin + 1;
    A.dmin = P.dmin;
    A.n_own = C;
    b200_dbuf d_own, d_in;
    if ((r = b200_alloc(n, d_own, (size_t)(C + 1) * 4, false))) return r;
    if ((r = b200_alloc(n, d_in, (size_t)C * 8))) return r;
    B200_CU(n, cudaMemcpyAsync(d_own.p, own_lo.data(), (size_t)(C + 1) * 4, cudaMemcpyHostToDevice, n->stream));
    A.own_lo = (const int32_t*)d_own.p;
    A.own_in = (unsigned long long*)d_in.p;
    A.oseg = (int64_t*)P.oseg.p;
    A.opost = (int32_t*)P.opost.p;
    A.odelay = (uint16_t*)P.odelay.p;
    A.status = (int32_t*)I.status.p;
    B200_CU(n, cudaMemsetAsync(I.status.p, 0, 4, n->stream));
    const int threads = 256, warps = threads / 32;
    const size_t smem = (size_t)((C + 1 + warps * C + 1) & ~1) * 4 + (size_t)warps * C * 8;
    if (smem > 48 * 1024)
      B200_CU(n, cudaFuncSetAttribute(b200_owner_relayout_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    int n_sm = 0, dev = 0;
    B200_CU(n, cudaGetDevice(&dev));
    B200_CU(n, cudaDeviceGetAttribute(&n_sm, cudaDevAttrMultiProcessorCount, dev));
    const int64_t want = (n_src + warps - 1) / warps;
    const int grid = (int)std::max<int64_t>(1, std::min<int64_t>(want, (int64_t)n_sm * 8));
    b200_owner_relayout_kernel<<<grid, threads, smem, n->stream>>>(A);
    B200_CU(n, cudaGetLastError());
    B200_CU(n, cudaStreamSynchronize(n->stream));
    b200_free(n, d_own);
    P.own_in.assign(C, 0);
    B200_CU(n, cudaMemcpy(P.own_in.data(), d_in.p, (size_t)C * 8, cudaMemcpyDeviceToHost));
    b200_free(n, d_in);
    int32_t st = 0;
    B200_CU(n, cudaMemcpy(&st, I.status.p, 4, cudaMemcpyDeviceToHost));
    if (st) {
      cudaMemset(I.status.p, 0, 4);
      return b200_fail(n, B200_ERR_INDEX, "pathway %s: a target lies outside the target group's tiles", PI.name);
    }
    P.own_lo = own_lo;
    P.own_stale = false;
  }
  // event FIFOs (pathways with delays), in records per CTA.  A synapse carries
  // at most one event per step and a batch is freed when its longest delay is
  // delivered, so dmax + 2 batches of the largest CTA's incoming synapses never
  // overflow: the default where that fits in an eighth of the device's memory,
  // else the largest power of two that does (at least one batch).  An explicit
  // b200_set_event_capacity factor sizes them in units of the incoming synapses.
  if (delays) {
    int64_t max_in = 1;
    for (int c = 0; c < C; ++c) max_in = std::max(max_in, P.own_in[c]);
    const int32_t W = P.dmax - P.dmin + 1, RB = P.dmax + 2;
    size_t rec = 4;
    for (int m = 0; m < PI.n_payload; ++m) rec += b200_kind_size(PI.var_kind[PI.payload_var[m]]);
    int64_t cap;
    if (n->ev_factor > 0) {
      cap = b200_pow2ceil(std::max<int64_t>((int64_t)(n->ev_factor * (double)max_in) + 1, (int64_t)1 << 10));
    } else {
      size_t free_b = 0, total_b = 0;
      B200_CU(n, cudaMemGetInfo(&free_b, &total_b));
      const int64_t floor_cap = b200_pow2ceil(std::max<int64_t>(max_in + 1, (int64_t)1 << 10));
      cap = b200_pow2ceil(std::max<int64_t>(max_in * (int64_t)(P.dmax + 2), (int64_t)1 << 10));
      while (cap > floor_cap && (double)C * (double)cap * (double)rec > (double)total_b / 8) cap >>= 1;
    }
    if (cap != P.ev_cap || W != P.ev_W || RB != P.ev_RB || C != P.ev_ncta) {
      if (I.ts > 0 && I.ran_owner == 1 && P.ev_cap > 0)
        return b200_fail(n, B200_ERR_ARG, "pathway %s: the event FIFO cannot be resized once the network has run", PI.name);
      if ((r = b200_alloc(n, P.ev_tgt, (size_t)C * cap * 4, false))) return r;
      P.ev_pay.resize(PI.n_payload);
      for (int m = 0; m < PI.n_payload; ++m)
        if ((r = b200_alloc(n, P.ev_pay[m], (size_t)C * cap * b200_kind_size(PI.var_kind[PI.payload_var[m]]), false)))
          return r;
      if ((r = b200_alloc(n, P.ev_state, (size_t)C * 2 * 8))) return r;
      if ((r = b200_alloc(n, P.ev_base, (size_t)C * RB * 8))) return r;
      if ((r = b200_alloc(n, P.ev_tag, (size_t)C * RB * 8, false))) return r;
      B200_CU(n, cudaMemsetAsync(P.ev_tag.p, 0xff, (size_t)C * RB * 8, n->stream));  // -1: no batch
      if ((r = b200_alloc(n, P.ev_off, (size_t)C * RB * (W + 1) * 4))) return r;
      B200_CU(n, cudaStreamSynchronize(n->stream));
      P.ev_cap = cap; P.ev_W = W; P.ev_RB = RB; P.ev_ncta = C;
    }
  }
  PD.segptr = (const int64_t*)P.oseg.p;
  PD.post = (const int32_t*)P.opost.p;
  PD.pre = nullptr;
  for (int v = 0; v < B200_MAX_VARS; ++v) PD.var[v] = nullptr;
  for (int m = 0; m < PI.n_payload; ++m) PD.var[PI.payload_var[m]] = P.ovar[m].p;
  PD.odelay = (const uint16_t*)P.odelay.p;
  memset(&PD.ev, 0, sizeof(PD.ev));
  if (!delays) { PD.D = 0; PD.dmin = 0; }  // no FIFO: a pathway without synapses has no events
  if (delays) {
    PD.ev.cap = P.ev_cap; PD.ev.RB = P.ev_RB; PD.ev.W = P.ev_W;
    PD.ev.tgt = (int32_t*)P.ev_tgt.p;
    for (int m = 0; m < PI.n_payload; ++m) PD.ev.pay[m] = P.ev_pay[m].p;
    PD.ev.state = (int64_t*)P.ev_state.p;
    PD.ev.base = (int64_t*)P.ev_base.p;
    PD.ev.tag = (int64_t*)P.ev_tag.p;
    PD.ev.off = (int32_t*)P.ev_off.p;
  }
  return 0;
}

static int b200_prepare(b200_net* n) {
  const b200_model_info* M = n->M;
  int r;
  // owner mode: a model whose on_pre code allows it, every instance on 2+ CTAs
  {
    bool want = n->allow_owner != 0 && M->owner_ok && !n->queue_mode;
    for (int k = 0; k < n->n_inst && want; ++k) want = n->inst[k].n_cta >= 2;
    // auto: owner mode where it is measured faster (no synaptic delays)
    for (int k = 0; k < n->n_inst && want && n->allow_owner == 2; ++k)
      for (int p = 0; p < M->n_pathways; ++p)
        if (n->inst[k].p[p].n_syn > 0 && n->inst[k].p[p].dmax > 0) want = false;
    // push mode: a model whose on_pre allows it, every synaptic delay >= 1 step;
    // auto: float32 models (the deliveries of a step are summed before they reach
    // their variable, which changes float64 results in the last bits) on 2+ CTAs
    bool push = n->allow_push != 0 && M->push_ok && !n->queue_mode;
    bool any_delay = false;
    for (int k = 0; k < n->n_inst && push; ++k)
      for (int p = 0; p < M->n_pathways; ++p) {
        if (n->inst[k].p[p].n_syn > 0 && n->inst[k].p[p].dmin == 0) push = false;
        if (n->inst[k].p[p].n_syn > 0 && n->inst[k].p[p].dmax > 0) any_delay = true;
      }
    if (push && n->allow_push == 2) {
      bool f32 = M->n_acc > 0;
      for (int a = 0; a < M->n_acc; ++a)
        f32 = f32 && M->groups[M->acc_vars[2 * a]].var_kind[M->acc_vars[2 * a + 1]] == B200_F32;
      push = f32 && any_delay;
      for (int k = 0; k < n->n_inst && push; ++k) push = n->inst[k].n_cta >= 2;
    }
    n->push = push ? 1 : 0;
    n->owner = (want && !push) ? 1 : 0;
    for (int k = 0; k < n->n_inst; ++k) {
      const b200_inst_h& I = n->inst[k];
      bool inflight = false;
      for (int p = 0; p < M->n_pathways; ++p) inflight = inflight || (I.p[p].dmax >= 1 && I.p[p].n_syn > 0);
      if (I.ts > 0 && inflight && I.ran_owner >= 0 && I.ran_owner != n->mode())
        return b200_fail(n, B200_ERR_ARG,
                         "instance %d: switching between the classic, owner and push delivery modes after the "
                         "first run of a network with delays would lose the spikes in flight; choose the mode "
                         "(b200_set_owner, b200_set_push) and the CTA count before the first run", k);
      if (n->push && I.ts > 0 && inflight && I.ran_owner == 2) {
        for (int g = 0; g < M->n_groups; ++g)
          if (I.g[g].hist_ncta != 0 && I.g[g].hist_ncta != I.n_cta)
            return b200_fail(n, B200_ERR_ARG,
                             "instance %d: the CTA count of a push-mode network with spikes in flight cannot "
                             "change between runs", k);
      }
    }
  }
  n->h_insts.assign(n->n_inst, b200_inst_d());
  std::vector<int2> cta_map;
  int cta = 0;
  for (int k = 0; k < n->n_inst; ++k) {
    b200_inst_h& I = n->inst[k];
    b200_inst_d& D = n->h_insts[k];
    memset(&D, 0, sizeof(D));
    D.n_cta = I.n_cta;
    D.cta0 = n->queue_mode ? 0 : cta;
    if (!n->queue_mode)
      for (int c = 0; c < I.n_cta; ++c) cta_map.push_back(make_int2(k, c));
    cta += I.n_cta;
    D.ts = I.ts;
    D.dt = n->dt;
    if ((r = b200_alloc(n, I.bar, 16))) return r;
    if ((r = b200_alloc(n, I.status, 16))) return r;
    if ((r = b200_alloc(n, I.ts_done, 16))) return r;
    if ((r = b200_alloc(n, I.pending, 16 * 4))) return r;
    D.bar = (unsigned*)I.bar.p;
    D.status = (int32_t*)I.status.p;
    D.ts_done = (int64_t*)I.ts_done.p;
    D.pending_reset = (int32_t*)I.pending.p;
    for (int g = 0; g < M->n_groups; ++g) {
      b200_group_h& G = I.g[g];
      std::vector<int32_t> cuts;
      int32_t R = 1;
      for (int p = 0; p < M->n_pathways; ++p)
        if (M->pathways[p].src_group == g) {
          cuts.push_back(I.p[p].src_lo);
          cuts.push_back(I.p[p].src_hi);
          R = std::max(R, I.p[p].dmax + 1);
        }
      for (int s = 0; s < M->n_spkmon; ++s)
        if (M->spkmon[s].group == g) { cuts.push_back(I.sm[s].lo); cuts.push_back(I.sm[s].hi); }
      for (int s = 0; s < M->n_ratemon; ++s)
        if (M->ratemon[s].group == g) { cuts.push_back(I.rm[s].lo); cuts.push_back(I.rm[s].hi); }
      if (n->owner || n->push) R = B200_OWNER_RING;  // lists of the last steps only (FIFOs / history)
      const std::vector<int32_t> old_tiles = G.tile_start;
      if (M->groups[g].generator) {
        // a spike generator emits in array order (not by neuron): all its tiles
        // belong to the first CTA, split only at source/monitor range boundaries
        std::vector<int32_t> one;
        b200_make_tiles(G.N, 1, cuts, G.tile_start, one);
        G.cta_tile.assign(I.n_cta + 1, (int32_t)G.tile_start.size() - 1);
        G.cta_tile[0] = 0;
      } else {
        b200_make_tiles(G.N, I.n_cta, cuts, G.tile_start, G.cta_tile);
      }
      const int n_tiles = (int)G.tile_start.size() - 1;
      const bool ring_changed = (R != G.R) || !G.ring.p;
      const bool retile = !n->owner && !n->push && !ring_changed && old_tiles != G.tile_start && I.ts > 0 && R > 1;
      G.R = R;
      if ((r = b200_alloc(n, G.d_tile_start, G.tile_start.size() * 4, false))) return r;
      if ((r = b200_alloc(n, G.d_cta_tile, G.cta_tile.size() * 4, false))) return r;
      B200_CU(n, cudaMemcpyAsync(G.d_tile_start.p, G.tile_start.data(), G.tile_start.size() * 4, cudaMemcpyHostToDevice, n->stream));
      B200_CU(n, cudaMemcpyAsync(G.d_cta_tile.p, G.cta_tile.data(), G.cta_tile.size() * 4, cudaMemcpyHostToDevice, n->stream));
      if ((r = b200_alloc(n, G.scratch, (size_t)std::max(G.N, 1) * 4, false))) return r;
      if ((r = b200_alloc(n, G.tile_cnt, (size_t)n_tiles * 4))) return r;
      if (ring_changed) {
        // the ring keeps spikes in flight across runs; it is only rebuilt when
        // its size changes (first run, or new delays)
        if ((r = b200_alloc(n, G.ring, (size_t)R * std::max(G.N, 1) * 4))) return r;
        if ((r = b200_alloc(n, G.ring_total, (size_t)R * 4))) return r;
      }
      if ((r = b200_alloc(n, G.ring_prefix, (size_t)R * (n_tiles + 1) * 4, ring_changed))) return r;
      if (retile) {
        // spikes still in flight were indexed by the old tiles: recount them
        std::vector<int32_t> tot(R), ring((size_t)R * G.N), pre((size_t)R * (n_tiles + 1));
        B200_CU(n, cudaMemcpy(tot.data(), G.ring_total.p, (size_t)R * 4, cudaMemcpyDeviceToHost));
        B200_CU(n, cudaMemcpy(ring.data(), G.ring.p, (size_t)R * G.N * 4, cudaMemcpyDeviceToHost));
        for (int s = 0; s < R; ++s) {
          const int32_t* a = ring.data() + (size_t)s * G.N;
          for (int u = 0; u <= n_tiles; ++u)
            pre[(size_t)s * (n_tiles + 1) + u] =
                (int32_t)(std::lower_bound(a, a + tot[s], G.tile_start[u]) - a);
        }
        B200_CU(n, cudaMemcpy(G.ring_prefix.p, pre.data(), pre.size() * 4, cudaMemcpyHostToDevice));
      }
      std::vector<double> S(std::max(M->groups[g].n_scalars, 1));
      M->eval_scalars(0, g, I.consts.data(), n->dt, S.data());
      if ((r = b200_alloc(n, G.S, S.size() * 8, false))) return r;
      B200_CU(n, cudaMemcpyAsync(G.S.p, S.data(), S.size() * 8, cudaMemcpyHostToDevice, n->stream));
      B200_CU(n, cudaStreamSynchronize(n->stream));
      b200_group_d& GD = D.g[g];
      GD.N = G.N; GD.R = R; GD.n_tiles = n_tiles;
      GD.own_off = -1;  // no shared copy of the CTA's own spike lists unless placed below
      GD.tile_start = (const int32_t*)G.d_tile_start.p;
      GD.cta_tile = (const int32_t*)G.d_cta_tile.p;
      GD.scratch = (int32_t*)G.scratch.p;
      GD.tile_cnt = (int32_t*)G.tile_cnt.p;
      GD.ring = (int32_t*)G.ring.p;
      GD.ring_total = (int32_t*)G.ring_total.p;
      GD.ring_prefix = (int32_t*)G.ring_prefix.p;
      GD.RH = 0; GD.HCAP = 0; GD.hist_off = 0; GD.hcnt_off = 0; GD.hist = nullptr; GD.hcnt = nullptr;
      if (n->push) {
        // each CTA's spike lists of the steps whose deliveries are still due
        int32_t RH = 2;
        for (int p = 0; p < M->n_pathways; ++p)
          if (M->pathways[p].src_group == g) RH = std::max(RH, I.p[p].dmax + 1);
        if (RH != G.RH || G.hist_ncta != I.n_cta || !G.hist.p || !G.hcnt.p) {
          if ((r = b200_alloc(n, G.hist, (size_t)RH * std::max(G.N, 1) * 4, false))) return r;
          if ((r = b200_alloc(n, G.hcnt, (size_t)RH * I.n_cta * 4))) return r;
          G.RH = RH;
          G.hist_ncta = I.n_cta;
        }
        GD.RH = RH;
        GD.hist = (int32_t*)G.hist.p;
        GD.hcnt = (int32_t*)G.hcnt.p;
      }
      const b200_group_h& GS = M->groups[g].alias >= 0 ? I.g[M->groups[g].alias] : G;  // (state owner)
      for (int v = 0; v < M->groups[g].n_vars; ++v) GD.var[v] = GS.var[v].p;
      GD.S = (const double*)G.S.p;
      if (M->groups[g].generator) {
        if (!G.gen_last.p) {  // no lists set: a generator without spikes
          if ((r = b200_alloc(n, G.gen_last, 16))) return r;
          if ((r = b200_alloc(n, G.gen_bins, 16))) return r;
          if ((r = b200_alloc(n, G.gen_index, 16))) return r;
        }
        GD.gen_bins = (const int32_t*)G.gen_bins.p;
        GD.gen_index = (const int32_t*)G.gen_index.p;
        GD.gen_n = G.gen_n;
        GD.gen_last = (int32_t*)G.gen_last.p;
        GD.gen_period = G.gen_period;
      }
    }
    for (int p = 0; p < M->n_pathways; ++p) {
      b200_pathway_h& P = I.p[p];
      const b200_pathway_info& PI = M->pathways[p];
      if (!P.has_syn) {
        // no synapses: an empty CSR over the whole source group
        std::vector<int32_t> none;
        if ((r = b200_set_synapses(n, k, p, 0, I.g[PI.src_group].N, 0, I.g[PI.tgt_group].N,
                                   none.data(), none.data(), nullptr, 0, 0)))
          return r;
      }
      b200_pathway_d& PD = D.p[p];
      const b200_group_h& SG = I.g[PI.src_group];
      PD.D = P.dmax;
      PD.src_lo = P.src_lo; PD.src_hi = P.src_hi;
      PD.tile_lo = (int)(std::lower_bound(SG.tile_start.begin(), SG.tile_start.end(), P.src_lo) - SG.tile_start.begin());
      PD.tile_hi = (int)(std::lower_bound(SG.tile_start.begin(), SG.tile_start.end(), P.src_hi) - SG.tile_start.begin());
      PD.dmin = P.dmin;
      PD.n_syn = P.n_syn;
      PD.segptr = (const int64_t*)P.segptr.p;
      PD.post = (const int32_t*)P.post.p;
      PD.pre = (const int32_t*)P.pre.p;
      if (PI.alias >= 0) {  // the shared synapses' variables, pre and post arrays are the owner's
        const b200_pathway_h& O = I.p[PI.alias];
        for (int v = 0; v < PI.n_vars; ++v) PD.var[v] = O.var[v].p;
        PD.sidx = (const int64_t*)P.sidx.p;
      } else {
        for (int v = 0; v < PI.n_vars; ++v) PD.var[v] = P.var[v].p;
        PD.sidx = nullptr;
      }
      std::vector<double> S(std::max(PI.n_scalars, 1));
      M->eval_scalars(1, p, I.consts.data(), n->dt, S.data());
      if ((r = b200_alloc(n, P.S, S.size() * 8, false))) return r;
      B200_CU(n, cudaMemcpyAsync(P.S.p, S.data(), S.size() * 8, cudaMemcpyHostToDevice, n->stream));
      B200_CU(n, cudaStreamSynchronize(n->stream));
      PD.S = (const double*)P.S.p;
      if (n->owner && (r = b200_owner_pathway(n, k, p, PD))) return r;
    }
    // every pathway with synapses has delays >= 1 step: a step's deliveries do
    // not read that step's spikes (owner mode pushes with a lag of one step,
    // classic mode prepares its deliveries while its barrier completes)
    D.lag = 1;
    for (int p = 0; p < M->n_pathways; ++p)
      if (I.p[p].n_syn > 0 && I.p[p].dmin == 0) D.lag = 0;
    if (n->owner) {
      D.owner = 1;
      if ((r = b200_alloc(n, I.bar64, 16))) return r;
      D.bar64 = (unsigned long long*)I.bar64.p;
    }
    if (n->push) {
      D.push = 1;
      if ((r = b200_alloc(n, I.bar64, 16))) return r;
      D.bar64 = (unsigned long long*)I.bar64.p;
      // the accumulators keep the deliveries due at the next steps across runs:
      // (re)allocated, zeroed, only when missing or too small
      for (int a = 0; a < M->n_acc; ++a) {
        const int ag = M->acc_vars[2 * a], av = M->acc_vars[2 * a + 1];
        const size_t bytes = (size_t)B200_PUSH_BUFS * std::max(I.g[ag].N, 1) * b200_kind_size(M->groups[ag].var_kind[av]);
        if (!I.acc[a].p || I.acc[a].bytes < bytes)
          if ((r = b200_alloc(n, I.acc[a], bytes))) return r;
        D.acc[a] = I.acc[a].p;
      }
    }
    for (int s = 0; s < M->n_spkmon; ++s) {
      b200_spkmon_h& S = I.sm[s];
      const b200_group_h& G = I.g[M->spkmon[s].group];
      if (!S.n.p) {
        if ((r = b200_alloc(n, S.n, 16))) return r;
        if ((r = b200_alloc(n, S.count, (size_t)std::max(S.hi - S.lo, 1) * 4))) return r;
      }
      const int nv = M->spkmon[s].n_vars;
      if (!S.i.p) {
        S.cap = std::max<int64_t>(1 << 16, 8 * (int64_t)(S.hi - S.lo));
        if ((r = b200_alloc(n, S.i, (size_t)S.cap * 4, false))) return r;
        if ((r = b200_alloc(n, S.ts, (size_t)S.cap * 4, false))) return r;
        if (nv > 0 && (r = b200_alloc(n, S.vals, (size_t)S.cap * nv * 8, false))) return r;
      }
      if (nv > 0 && (r = b200_alloc(n, S.snap, (size_t)nv * std::max(G.N, 1) * 8))) return r;
      b200_spkmon_d& SD = D.sm[s];
      SD.group = M->spkmon[s].group; SD.lo = S.lo; SD.hi = S.hi;
      SD.n_vars = nv;
      SD.snap = (double*)S.snap.p; SD.vals = (double*)S.vals.p;
      SD.tile_lo = (int)(std::lower_bound(G.tile_start.begin(), G.tile_start.end(), S.lo) - G.tile_start.begin());
      SD.tile_hi = (int)(std::lower_bound(G.tile_start.begin(), G.tile_start.end(), S.hi) - G.tile_start.begin());
      SD.cap = S.cap;
      SD.n = (int64_t*)S.n.p; SD.i = (int32_t*)S.i.p; SD.ts = (int32_t*)S.ts.p;
      SD.count = (int32_t*)S.count.p;
      SD.xcnt = nullptr;
      if (n->push) {
        if ((r = b200_alloc(n, S.xcnt, (size_t)3 * I.n_cta * 4))) return r;
        SD.xcnt = (int32_t*)S.xcnt.p;
      }
    }
    for (int s = 0; s < M->n_ratemon; ++s) {
      b200_ratemon_h& S = I.rm[s];
      const b200_group_h& G = I.g[M->ratemon[s].group];
      b200_ratemon_d& RD = D.rm[s];
      RD.group = M->ratemon[s].group; RD.lo = S.lo; RD.hi = S.hi;
      RD.tile_lo = (int)(std::lower_bound(G.tile_start.begin(), G.tile_start.end(), S.lo) - G.tile_start.begin());
      RD.tile_hi = (int)(std::lower_bound(G.tile_start.begin(), G.tile_start.end(), S.hi) - G.tile_start.begin());
      RD.xcnt = nullptr;
      if (n->push) {
        if ((r = b200_alloc(n, S.xcnt, (size_t)3 * I.n_cta * 4))) return r;
        RD.xcnt = (int32_t*)S.xcnt.p;
      }
    }
    for (int s = 0; s < M->n_statemon; ++s) {
      b200_statemon_h& S = I.stm[s];
      b200_statemon_d& SD = D.stm[s];
      SD.group = M->statemon[s].group;
      SD.n_rec = S.n_rec;
      SD.n_vars = S.n_vars;
      if ((r = b200_alloc(n, S.d_idx, (size_t)std::max(S.n_rec, 1) * 4, false))) return r;
      const int sp = M->statemon[s].syn;
      std::vector<int32_t> rec(S.idx);
      if (sp >= 0 && S.n_rec) {  // synapse index -> its position in the synapses' CSR order
        const b200_pathway_h& P = I.p[sp];
        if (P.n_syn > INT32_MAX) return b200_fail(n, B200_ERR_ARG, "state monitor of more than 2^31 synapses");
        std::vector<int32_t> inv((size_t)P.n_syn);
        for (int64_t q = 0; q < P.n_syn; ++q) inv[(size_t)P.perm[q]] = (int32_t)q;
        for (auto& x : rec) {
          if (x < 0 || x >= P.n_syn) return b200_fail(n, B200_ERR_INDEX, "state monitor %d: no synapse %d", s, x);
          x = inv[(size_t)x];
        }
      }
      if (S.n_rec)
        B200_CU(n, cudaMemcpyAsync(S.d_idx.p, rec.data(), (size_t)S.n_rec * 4, cudaMemcpyHostToDevice, n->stream));
      B200_CU(n, cudaStreamSynchronize(n->stream));
      if (!S.n.p && (r = b200_alloc(n, S.n, 16))) return r;
      SD.idx = (const int32_t*)S.d_idx.p;
      for (int v = 0; v < S.n_vars; ++v) {
        SD.var_id[v] = S.vars[v];
        SD.var_dbl[v] = (sp >= 0 ? M->pathways[sp].var_kind[S.vars[v]] : M->groups[SD.group].var_kind[S.vars[v]]) ==
                        B200_F64;
      }
      SD.n = (int64_t*)S.n.p;
    }
    for (int sv = 0; sv < M->n_summed; ++sv) {  // (the pathways' synapses are set above)
      const b200_summed_h& S = I.sum[sv];
      D.sum[sv].lo = S.lo; D.sum[sv].hi = S.hi;
      D.sum[sv].seg = (const int64_t*)S.seg.p;
      D.sum[sv].syn = (const int64_t*)S.syn.p;
    }
  }
  n->max_tiles1 = 2;
  n->max_w = 1;
  for (int k = 0; k < n->n_inst; ++k) {
    for (int g = 0; g < M->n_groups; ++g)
      n->max_tiles1 = std::max(n->max_tiles1, (int)n->inst[k].g[g].tile_start.size());
    // pathways of one source may share a delivery pass: their delay windows add up
    int wsum = 0;
    for (int p = 0; p < M->n_pathways; ++p) wsum += n->inst[k].p[p].dmax - n->inst[k].p[p].dmin + 1;
    n->max_w = std::max(n->max_w, wsum);
  }
  // shared-memory state cache of single-CTA instances: the used state
  // variables, the step's spike list and the tile counts
  {
    int dev = 0, optin = 0;
    B200_CU(n, cudaGetDevice(&dev));
    B200_CU(n, cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev));
    // sweeps with more instances than SMs use the two-CTAs-per-SM variant
    int n_sm_ = 0, dev_ = 0;
    B200_CU(n, cudaGetDevice(&dev_));
    B200_CU(n, cudaDeviceGetAttribute(&n_sm_, cudaDevAttrMultiProcessorCount, dev_));
    // instances on more CTAs than SMs (two per SM, so one CTA's barrier waits overlap
    // the other's work) use it too
    int max_cta = 0;
    for (int k = 0; k < n->n_inst; ++k) max_cta = std::max(max_cta, n->inst[k].n_cta);
    n->min_blocks = (!n->owner && ((n->threads == 512 && n->queue_mode && n->n_inst > n_sm_ && !n->push) ||
                                   ((n->threads == 512 || n->threads == 256) && !n->queue_mode && max_cta > n_sm_)))
                        ? 2 : 1;
    const long other = (long)M->static_smem(n->tcode()) +
                       (long)(n->threads * 20 + 4 + 2 * M->n_groups * n->max_tiles1 * 4 + (3 * n->max_w + 1) * 4 + 64) +
                       (n->owner ? (long)n->max_w * 8 + (long)(n->max_w + 1) * 4 : 0L);
    const long budget = (long)optin - other - 1024;
    // bytes of the cache of instance k: state variables, plus (lists) the step's
    // spike list and tile counts
    auto cache_bytes = [&](int k, bool lists) -> long {
      b200_inst_h& I = n->inst[k];
      if (!n->smem_cache) return 0;
      if (n->owner || n->push) {  // each CTA caches the neurons it owns
        long worst = 0;
        for (int c = 0; c < I.n_cta; ++c) {
          long bytes = 0;
          for (int g = 0; g < M->n_groups; ++g) {
            const b200_group_h& G = I.g[g];
            const long Ng = G.tile_start[G.cta_tile[c + 1]] - G.tile_start[G.cta_tile[c]];
            for (int v = 0; v < M->groups[g].n_vars; ++v)
              if (M->groups[g].var_used[v]) bytes += (Ng * (long)b200_kind_size(M->groups[g].var_kind[v]) + 15) & ~15L;
          }
          worst = std::max(worst, bytes);
        }
        return worst > budget ? 0 : worst;
      }
      if (I.n_cta != 1) return 0;
      long bytes = 0;
      for (int g = 0; g < M->n_groups; ++g) {
        const long Ng = I.g[g].N;
        for (int v = 0; v < M->groups[g].n_vars; ++v)
          if (M->groups[g].var_used[v]) bytes += (Ng * (long)b200_kind_size(M->groups[g].var_kind[v]) + 15) & ~15L;
        if (lists) {
          bytes += (Ng * 4 + 15) & ~15L;
          bytes += ((long)(I.g[g].tile_start.size() - 1) * 4 + 15) & ~15L;
        }
      }
      return bytes > budget ? 0 : bytes;
    };
    long with_lists = 0, state_only = 0;
    for (int k = 0; k < n->n_inst; ++k) {
      with_lists = std::max(with_lists, cache_bytes(k, true));
      state_only = std::max(state_only, cache_bytes(k, false));
    }
    // a sweep of many instances wants two resident CTAs per SM: drop the lists
    // from the cache when that is what it takes
    bool lists = true;
    if (n->queue_mode && n->n_inst > 1) {
      const long half = (long)optin / 2 - other - 1024;
      if (with_lists > half && state_only <= half) lists = false;
    }
    n->state_bytes = 0;
    for (int k = 0; k < n->n_inst; ++k) {
      const long bytes = cache_bytes(k, lists);
      n->h_insts[k].cache_bytes = (int32_t)bytes;
      n->h_insts[k].cache_lists = lists ? 1 : 0;
      n->state_bytes = std::max<long>(n->state_bytes, bytes);
    }
    if (!n->owner && !n->push && !n->queue_mode) {
      // classic multi-CTA instances: each CTA keeps its own neurons' private
      // variables (touched by no pathway) in shared memory for the launch, then
      // a copy of its own spike lists and tile counts (the reset and the ring
      // copy read them there); with two CTAs per SM each gets half the room
      const long room = n->min_blocks == 2 ? std::min(budget, (long)optin / 2 - other - 1024) : budget;
      for (int k = 0; k < n->n_inst; ++k) {
        b200_inst_d& D = n->h_insts[k];
        if (D.cache_bytes > 0) continue;
        const b200_inst_h& I = n->inst[k];
        long priv = 0;
        if (n->smem_cache && I.n_cta > 1) {
          for (int c = 0; c < I.n_cta; ++c) {
            long b = 0;
            for (int g = 0; g < M->n_groups; ++g) {
              const b200_group_h& G = I.g[g];
              const long Ng = G.tile_start[G.cta_tile[c + 1]] - G.tile_start[G.cta_tile[c]];
              for (int v = 0; v < M->groups[g].n_vars; ++v)
                if (M->groups[g].var_private[v]) b += (Ng * (long)b200_kind_size(M->groups[g].var_kind[v]) + 15) & ~15L;
            }
            priv = std::max(priv, b);
          }
          if (priv > room) priv = 0;
        }
        D.priv_bytes = (int32_t)priv;
        n->state_bytes = std::max<long>(n->state_bytes, priv);
        long off = (priv + 15) & ~15L;
        std::vector<long> offs(M->n_groups);
        for (int g = 0; g < M->n_groups; ++g) {
          const b200_group_h& G = I.g[g];
          if (M->groups[g].generator) {  // all on the first CTA: global lists
            D.g[g].own_cap = 1; D.g[g].own_tiles = 1; offs[g] = -1;
            continue;
          }
          int cap = 0, tiles = 0;
          for (int c = 0; c < I.n_cta; ++c) {
            cap = std::max(cap, G.tile_start[G.cta_tile[c + 1]] - G.tile_start[G.cta_tile[c]]);
            tiles = std::max(tiles, G.cta_tile[c + 1] - G.cta_tile[c]);
          }
          D.g[g].own_cap = std::max(cap, 1);
          D.g[g].own_tiles = std::max(tiles, 1);
          offs[g] = off;
          off += (((long)D.g[g].own_cap * 4 + 15) & ~15L) + (((long)D.g[g].own_tiles * 4 + 15) & ~15L);
        }
        if (off <= room) {
          for (int g = 0; g < M->n_groups; ++g) D.g[g].own_off = (int32_t)offs[g];
          n->state_bytes = std::max<long>(n->state_bytes, off);
        }
      }
    }
    if (n->owner) {
      // after the state cache: the batch tables of the event FIFOs, then a
      // staging area for one step's events (one pass over the synapses)
      int total_cta = 0, n_sm_o = 0, dev_o = 0;
      for (int k = 0; k < n->n_inst; ++k) total_cta += n->inst[k].n_cta;
      B200_CU(n, cudaGetDevice(&dev_o));
      B200_CU(n, cudaDeviceGetAttribute(&n_sm_o, cudaDevAttrMultiProcessorCount, dev_o));
      const long room = total_cta > n_sm_o ? std::min(budget, (long)optin / 2 - other - 1024) : budget;
      for (int k = 0; k < n->n_inst; ++k) {
        b200_inst_d& D = n->h_insts[k];
        long off = ((long)D.cache_bytes + 15) & ~15L;
        long tab = 0;
        for (int p = 0; p < M->n_pathways; ++p)
          if (D.p[p].ev.cap > 0)
            tab += (((long)D.p[p].ev.RB * (D.p[p].ev.W + 1) * 4 + 15) & ~15L) + (long)D.p[p].ev.RB * 16;
        D.tab_smem = (tab > 0 && off + tab <= room) ? 1 : 0;
        if (D.tab_smem)
          for (int p = 0; p < M->n_pathways; ++p)
            if (D.p[p].ev.cap > 0) {
              D.p[p].ev.tab_off = (int32_t)off;
              off += (((long)D.p[p].ev.RB * (D.p[p].ev.W + 1) * 4 + 15) & ~15L) + (long)D.p[p].ev.RB * 16;
            }
        const long ev = std::max(8, M->owner_event_bytes);
        // staging only serves pathways with delays (the others deliver at once)
        long cap = (tab > 0 && off < room) ? std::min<long>(16384, (room - off) / ev) : 0;
        cap &= ~3L;
        D.stage_off = (int32_t)off;
        D.stage_cap = (int32_t)cap;
        off += cap * ev;
        n->state_bytes = std::max<long>(n->state_bytes, off);
      }
    }
    if (n->push) {
      // after the state cache: per group the slot counts of the spike history and
      // its first HCAP entries per slot, per pathway the bounds of its source
      // range per slot (HCAP as large as the room allows, at most 64)
      const long room = n->min_blocks == 2 ? std::min(budget, (long)optin / 2 - other - 1024) : budget;
      for (int k = 0; k < n->n_inst; ++k) {
        b200_inst_d& D = n->h_insts[k];
        long off = ((long)D.cache_bytes + 15) & ~15L;
        long hist_words = 0;
        const b200_inst_h& IH = n->inst[k];
        for (int g = 0; g < M->n_groups; ++g) {
          D.g[g].hcnt_off = (int32_t)off;
          off += ((long)D.g[g].RH * 4 + 15) & ~15L;
          hist_words += D.g[g].RH;
          // each warp's spikes of the step, in neuron order, before they enter the history
          int cap = 0;
          const b200_group_h& G = IH.g[g];
          for (int c = 0; c < IH.n_cta; ++c) cap = std::max(cap, G.tile_start[G.cta_tile[c + 1]] - G.tile_start[G.cta_tile[c]]);
          D.g[g].own_cap = cap + 128 * (n->threads / 32);
          D.g[g].own_off = (int32_t)off;
          off += ((long)D.g[g].own_cap * 4 + 15) & ~15L;
        }
        for (int p = 0; p < M->n_pathways; ++p) {
          D.p[p].pb_off = (int32_t)off;
          off += (long)D.g[M->pathways[p].src_group].RH * 8;
        }
        long hcap = hist_words > 0 ? std::min<long>(64, std::max<long>(0, room - off - 16 * M->n_groups) / (hist_words * 4)) : 0;
        if (hcap < 0) hcap = 0;
        for (int g = 0; g < M->n_groups; ++g) {
          D.g[g].HCAP = (int32_t)hcap;
          D.g[g].hist_off = (int32_t)off;
          off += ((long)D.g[g].RH * hcap * 4 + 15) & ~15L;
        }
        n->state_bytes = std::max<long>(n->state_bytes, off);
      }
    }
  }
  int max_per_sm = M->max_active_ctas(n->tcode(), n->max_tiles1, n->max_w, n->state_bytes);
  int dev = 0, n_sm = 0;
  B200_CU(n, cudaGetDevice(&dev));
  B200_CU(n, cudaDeviceGetAttribute(&n_sm, cudaDevAttrMultiProcessorCount, dev));
  const int resident = std::max(1, max_per_sm) * n_sm;
  // thread-block clusters: every instance has the same CTA count C in 2..16
  n->cluster = 0;
  if (!n->queue_mode && n->use_clusters && n->fault_rank < 0) {
    int C = n->inst[0].n_cta;
    bool same = true;
    for (int k = 1; k < n->n_inst; ++k) same = same && n->inst[k].n_cta == C;
    if (same && C >= 2 && C <= 16 &&
        M->max_cluster(n->tcode(), n->max_tiles1, n->max_w, n->state_bytes, C) >= C)
      n->cluster = C;
  }
  if (n->queue_mode) {
    n->grid = std::min(n->n_inst, resident);
  } else if (n->cluster) {
    n->grid = cta;  // independent clusters: no co-residency of the whole grid needed
  } else {
    n->grid = cta;
    if (cta > resident)
      return b200_fail(n, B200_ERR_ARG,
                       "%d CTAs requested but only %d can be resident (%d/SM); use queue mode or fewer CTAs",
                       cta, resident, max_per_sm);
  }
  if ((r = b200_alloc(n, n->d_cta_map, std::max<size_t>(cta_map.size(), 1) * sizeof(int2), false))) return r;
  if (!cta_map.empty())
    B200_CU(n, cudaMemcpyAsync(n->d_cta_map.p, cta_map.data(), cta_map.size() * sizeof(int2), cudaMemcpyHostToDevice, n->stream));
  if ((r = b200_alloc(n, n->d_work, 16))) return r;
  if ((r = b200_alloc(n, n->d_insts, sizeof(b200_inst_d) * n->n_inst, false))) return r;
  B200_CU(n, cudaStreamSynchronize(n->stream));
  if (n->graph_exec) {
    cudaGraphExecDestroy(n->graph_exec);
    n->graph_exec = nullptr;
    n->graph_steps = -1;
  }
  n->prepared = true;
  return 0;
}

// Grow a spike monitor (nv recorded variables) so that at least `need` more spikes fit.
static int b200_grow_spkmon(b200_net* n, b200_spkmon_h& S, int nv, int64_t used, int64_t need) {
  int64_t cap = S.cap;
  while (cap - used < need) cap *= 2;
  if (cap == S.cap) return 0;
  b200_dbuf ni, nt, nvl;
  int r;
  if ((r = b200_alloc(n, ni, (size_t)cap * 4, false))) return r;
  if ((r = b200_alloc(n, nt, (size_t)cap * 4, false))) return r;
  if (nv > 0 && (r = b200_alloc(n, nvl, (size_t)cap * nv * 8, false))) return r;
  if (used) {
    B200_CU(n, cudaMemcpyAsync(ni.p, S.i.p, (size_t)used * 4, cudaMemcpyDeviceToDevice, n->stream));
    B200_CU(n, cudaMemcpyAsync(nt.p, S.ts.p, (size_t)used * 4, cudaMemcpyDeviceToDevice, n->stream));
    if (nv > 0)
      B200_CU(n, cudaMemcpyAsync(nvl.p, S.vals.p, (size_t)used * nv * 8, cudaMemcpyDeviceToDevice, n->stream));
  }
  B200_CU(n, cudaStreamSynchronize(n->stream));
  b200_free(n, S.i);
  b200_free(n, S.ts);
  S.i = ni;
  S.ts = nt;
  if (nv > 0) {
    b200_free(n, S.vals);
    S.vals = nvl;
  }
  S.cap = cap;
  return 0;
}

extern "C" {

// Runs every instance for n_steps time steps from its current step.  Replaces
// Network::run (brian2/devices/cpp_standalone/templates/network.cpp:38-122):
// the per-step schedule runs on the device inside the persistent kernel, the
// host only relaunches when a spike monitor needs more room.
int b200_run(b200_net* n, int64_t n_steps) {
  if (!n) return B200_ERR_ARG;
  if (n_steps < 0) return b200_fail(n, B200_ERR_ARG, "negative step count");
  for (int k = 0; k < n->n_inst; ++k)
    if (n->inst[k].stale)
      return b200_fail(n, B200_ERR_ARG,
                       "instance %d: an earlier run failed part-way, so its state belongs to no single time "
                       "step; upload the state and call b200_set_step before running it again", k);
  int r;
  if (!n->prepared && (r = b200_prepare(n))) return r;
  const b200_model_info* M = n->M;
  // rate / state monitors get room for the whole run up front
  for (int k = 0; k < n->n_inst; ++k) {
    b200_inst_h& I = n->inst[k];
    for (int s = 0; s < M->n_ratemon; ++s) {
      b200_ratemon_h& S = I.rm[s];
      const int64_t need = I.ts + n_steps - S.step0;
      if (S.cap < need) {
        b200_dbuf nb;
        const int64_t cap = std::max<int64_t>(need, 2 * S.cap);
        if ((r = b200_alloc(n, nb, (size_t)cap * 4))) return r;
        if (S.cap) B200_CU(n, cudaMemcpyAsync(nb.p, S.cnt.p, (size_t)S.cap * 4, cudaMemcpyDeviceToDevice, n->stream));
        B200_CU(n, cudaStreamSynchronize(n->stream));
        b200_free(n, S.cnt);
        S.cnt = nb;
        S.cap = cap;
      }
      n->h_insts[k].rm[s].step0 = S.step0;
      n->h_insts[k].rm[s].cap = S.cap;
      n->h_insts[k].rm[s].cnt = (int32_t*)S.cnt.p;
    }
    for (int s = 0; s < M->n_statemon; ++s) {
      b200_statemon_h& S = I.stm[s];
      // rows through the last step of this run: one per step whose index is a
      // multiple of the monitor's period, from step0 on
      const int64_t ev = std::max(M->statemon[s].every, 1);
      const int64_t need = std::max<int64_t>((I.ts + n_steps - 1) / ev - (S.step0 + ev - 1) / ev + 1, 0);
      const size_t row = (size_t)std::max(S.n_rec * S.n_vars, 1) * 8;
      if (S.cap < need) {
        b200_dbuf nb;
        const int64_t cap = std::max<int64_t>(need, 2 * S.cap);
        if ((r = b200_alloc(n, nb, (size_t)cap * row))) return r;
        if (S.cap) B200_CU(n, cudaMemcpyAsync(nb.p, S.data.p, (size_t)S.cap * row, cudaMemcpyDeviceToDevice, n->stream));
        B200_CU(n, cudaStreamSynchronize(n->stream));
        b200_free(n, S.data);
        S.data = nb;
        S.cap = cap;
      }
      n->h_insts[k].stm[s].step0 = S.step0;
      n->h_insts[k].stm[s].cap = S.cap;
      n->h_insts[k].stm[s].data = (double*)S.data.p;
    }
  }
  std::vector<int64_t> target(n->n_inst);
  for (int k = 0; k < n->n_inst; ++k) target[k] = n->inst[k].ts + n_steps;
  cudaEvent_t e0, e1;
  B200_CU(n, cudaEventCreate(&e0));
  B200_CU(n, cudaEventCreate(&e1));
  B200_CU(n, cudaEventRecord(e0, n->stream));
  const int coop = (!n->queue_mode && !n->cluster) ? 1 : 0;
  cudaEvent_t k0, k1;
  B200_CU(n, cudaEventCreate(&k0));
  B200_CU(n, cudaEventCreate(&k1));
  double kernel_ms = 0.0;
  for (int guard = 0; guard < 1 << 20; ++guard) {
    bool any = false;
    for (int k = 0; k < n->n_inst; ++k) {
      b200_inst_h& I = n->inst[k];
      b200_inst_d& D = n->h_insts[k];
      D.ts = I.ts;
      D.ts_end = target[k];
      if (I.ts < target[k]) any = true;
      for (int s = 0; s < M->n_spkmon; ++s) {
        b200_spkmon_h& S = I.sm[s];
        int64_t used = 0;
        B200_CU(n, cudaMemcpy(&used, S.n.p, 8, cudaMemcpyDeviceToHost));
        // room for at least 64 steps of all neurons spiking
        // (owner mode records a step's spikes one step later: one more step of room)
        const int64_t need = (std::min<int64_t>(target[k] - I.ts, 64) + ((n->owner || n->push) ? 1 : 0)) * (int64_t)(S.hi - S.lo);
        if ((r = b200_grow_spkmon(n, S, M->spkmon[s].n_vars, used, need))) return r;
        D.sm[s].cap = S.cap;
        D.sm[s].i = (int32_t*)S.i.p;
        D.sm[s].ts = (int32_t*)S.ts.p;
        D.sm[s].vals = (double*)S.vals.p;
      }
    }
    if (!any) break;
    int64_t steps = n->chunk_steps;
    if (M->n_draws > 0) {
      // the draws of the launch's steps, continuing the generator, in the order
      // of the draw sites (the reference's schedule)
      auto site_count = [&](const b200_inst_h& I, int q) -> int64_t {
        const b200_draw_info& D = M->draws[q];
        return ((D.hi < 0 ? (int64_t)I.g[D.group].N : (int64_t)D.hi) - D.lo) * D.calls;
      };
      int64_t per_step = 0;
      for (int q = 0; q < M->n_draws; ++q) per_step += site_count(n->inst[0], q);
      steps = std::max<int64_t>(1, std::min<int64_t>(steps, ((int64_t)128 << 20) / 8 / std::max<int64_t>(per_step, 1)));
      for (int k = 0; k < n->n_inst; ++k) {
        b200_inst_h& I = n->inst[k];
        b200_inst_d& Dd = n->h_insts[k];
        if (!I.rng_set) return b200_fail(n, B200_ERR_ARG, "instance %d: the model draws random numbers; set the generator (b200_set_rng)", k);
        b200_sites_d sites = {};
        sites.n_sites = M->n_draws;
        int64_t pk = 0;
        for (int q = 0; q < M->n_draws; ++q) {
          const b200_draw_info& D = M->draws[q];
          const int64_t c = site_count(I, q);
          if (D.lo < 0 || c < 0 || D.lo + c / std::max(D.calls, 1) > I.g[D.group].N)
            return b200_fail(n, B200_ERR_ARG, "instance %d: draw site '%s' covers neurons outside its group", k, D.name);
          Dd.draw_off[q] = (int32_t)pk;
          b200_site_d& S = sites.s[q];
          S.kind = D.kind; S.count = (int32_t)c; S.n = D.n; S.reverse = D.reverse;
          S.qn = D.qn; S.bound = D.bound; S.p = D.p; S.q = D.q; S.scale = D.scale; S.loc = D.loc;
          pk += c;
        }
        if (pk > INT32_MAX) return b200_fail(n, B200_ERR_ARG, "instance %d: too many draws per step", k);
        Dd.rng_per_step = (int32_t)pk;
        const int64_t w_k = std::max<int64_t>(pk, 1);
        const int64_t end = std::min<int64_t>(target[k], I.ts + steps);
        if (I.rng_from > I.ts || I.rng_to < I.ts)
          return b200_fail(n, B200_ERR_ARG, "instance %d: random stream position lost", k);
        if (end > I.rng_to) {
          // move the draws still unused to the other buffer, draw the rest after them
          const int nb = 1 - I.rng_cur;
          const int64_t keep = I.rng_to - I.ts;
          if ((r = b200_alloc(n, I.rng_buf[nb], (size_t)std::max<int64_t>(end - I.ts, 1) * w_k * 8, false))) return r;
          if (keep > 0)
            B200_CU(n, cudaMemcpyAsync(I.rng_buf[nb].p, (double*)I.rng_buf[I.rng_cur].p + (I.ts - I.rng_from) * w_k,
                                       (size_t)keep * w_k * 8, cudaMemcpyDeviceToDevice, n->stream));
          b200_variates_kernel<<<1, 1024, 0, n->stream>>>((uint32_t*)I.rng_state.p, (double*)I.rng_gauss.p, sites,
                                                          (double*)I.rng_buf[nb].p + keep * w_k, pk, end - I.rng_to,
                                                          (int32_t*)I.status.p);
          B200_CU(n, cudaGetLastError());
          I.rng_cur = nb;
          I.rng_from = I.ts;
          I.rng_to = end;
        }
        Dd.rng_vals = (const double*)I.rng_buf[I.rng_cur].p + (I.ts - I.rng_from) * w_k;
        Dd.rng_ts0 = I.ts;
      }
    }
    if (n->owner || n->push) {  // the split barrier counts the arrivals of this launch from 0
      for (int k = 0; k < n->n_inst; ++k) {
        n->h_insts[k].ts_base = n->inst[k].ts;
        B200_CU(n, cudaMemsetAsync(n->inst[k].bar64.p, 0, 8, n->stream));
      }
    }
    B200_CU(n, cudaMemcpyAsync(n->d_insts.p, n->h_insts.data(), sizeof(b200_inst_d) * n->n_inst,
                               cudaMemcpyHostToDevice, n->stream));
    B200_CU(n, cudaMemsetAsync(n->d_work.p, 0, 16, n->stream));

    B200_CU(n, cudaEventRecord(k0, n->stream));
    cudaError_t le = cudaSuccess;
    const bool graph = n->use_graph && n->fault_rank < 0;
    if (graph && (!n->graph_exec || n->graph_steps != steps)) {
      // capture the launch (work-queue reset + persistent kernel) once; every
      // later chunk is one graph replay
      if (n->graph_exec) {
        cudaGraphExecDestroy(n->graph_exec);
        n->graph_exec = nullptr;
      }
      cudaGraph_t g = nullptr;
      B200_CU(n, cudaStreamBeginCapture(n->stream, cudaStreamCaptureModeThreadLocal));
      cudaMemsetAsync(n->d_work.p, 0, 16, n->stream);
      le = M->launch((b200_inst_d*)n->d_insts.p, (const int2*)n->d_cta_map.p, n->n_inst, n->queue_mode,
                     (int*)n->d_work.p, steps, n->limit_ns, n->grid, n->tcode(), coop, n->max_tiles1,
                     n->max_w, n->fault_rank, n->state_bytes,
                     n->profiling ? (unsigned long long*)n->prof.p : nullptr, n->cluster, n->stream);
      cudaError_t ce = cudaStreamEndCapture(n->stream, &g);
      if (le != cudaSuccess || ce != cudaSuccess) {
        if (g) cudaGraphDestroy(g);
        cudaGetLastError();
        return b200_fail(n, B200_ERR_CUDA, "graph capture of the step launch: %s",
                         cudaGetErrorString(le != cudaSuccess ? le : ce));
      }
      le = cudaGraphInstantiate(&n->graph_exec, g, 0);
      cudaGraphDestroy(g);
      if (le != cudaSuccess) return b200_fail(n, B200_ERR_CUDA, "graph instantiate: %s", cudaGetErrorString(le));
      n->graph_steps = steps;
    }
    if (graph) {
      le = cudaGraphLaunch(n->graph_exec, n->stream);
    } else {
      le = M->launch((b200_inst_d*)n->d_insts.p, (const int2*)n->d_cta_map.p, n->n_inst,
                     n->queue_mode, (int*)n->d_work.p, steps, n->limit_ns, n->grid,
                     n->tcode(), coop, n->max_tiles1, n->max_w, n->fault_rank, n->state_bytes,
                     n->profiling ? (unsigned long long*)n->prof.p : nullptr,
                     n->cluster, n->stream);
    }
    if (n->fault_rank >= 0) {  // one-shot; the next launch may use clusters again
      n->fault_rank = -1;
      n->prepared = false;
    }
    if (le != cudaSuccess) return b200_fail(n, B200_ERR_CUDA, "kernel launch: %s", cudaGetErrorString(le));
    ++n->launches;
    B200_CU(n, cudaEventRecord(k1, n->stream));
    B200_CU(n, cudaStreamSynchronize(n->stream));
    {
      float kms = 0.f;
      cudaEventElapsedTime(&kms, k0, k1);
      kernel_ms += kms;
    }
    // read every instance's status first and clear the failed ones' status and
    // barrier words, so that one failure leaves no other instance with a
    // half-counted barrier; then report the first failure
    int first_bad = -1;
    int32_t bad_st = 0;
    int64_t bad_done = 0;
    for (int k = 0; k < n->n_inst; ++k) {
      b200_inst_h& I = n->inst[k];
      int32_t st = 0;
      int64_t done = 0;
      B200_CU(n, cudaMemcpy(&st, I.status.p, 4, cudaMemcpyDeviceToHost));
      B200_CU(n, cudaMemcpy(&done, I.ts_done.p, 8, cudaMemcpyDeviceToHost));
      if (st != 0) {
        B200_CU(n, cudaMemset(I.status.p, 0, 4));
        B200_CU(n, cudaMemset(I.bar.p, 0, 16));
        I.ts = done;
        // a binomial restart stops every CTA at the same step boundary; the
        // other failures leave CTAs at different steps
        if (st != B200_ERR_RANDOM) I.stale = true;
        if (first_bad < 0) { first_bad = k; bad_st = st; bad_done = done; }
        continue;
      }
      if (done < I.ts || done > target[k])
        return b200_fail(n, B200_ERR_CUDA, "instance %d: bad progress %lld", k, (long long)done);
      if (done > I.ts) I.ran_owner = n->mode();
      I.ts = done;
    }
    if (first_bad >= 0) {
      const int k = first_bad;
      if (bad_st == B200_ERR_RANDOM)
        return b200_fail(n, B200_STATUS_RANDOM_H,
                         "instance %d: a binomial draw before step %lld started over more often than the "
                         "stream's window holds numbers", k, (long long)bad_done);
      if (bad_st == B200_ERR_EVENT_OVERFLOW)
        return b200_fail(n, B200_ERR_CAPACITY,
                         "instance %d: an owner-mode event FIFO overflowed before step %lld (events were dropped; "
                         "raise its size with b200_set_event_capacity and run again from the start)",
                         k, (long long)bad_done);
      return b200_fail(n, bad_st == B200_ERR_BARRIER_TIMEOUT ? B200_ERR_BARRIER_TIMEOUT : B200_ERR_INDEX,
                       "instance %d: device status %d at step %lld (%s)", k, bad_st, (long long)bad_done,
                       bad_st == B200_ERR_BARRIER_TIMEOUT ? "instance barrier timed out" : "index out of range");
    }
  }
  B200_CU(n, cudaEventRecord(e1, n->stream));
  B200_CU(n, cudaEventSynchronize(e1));
  float ms = 0;
  cudaEventElapsedTime(&ms, e0, e1);
  n->last_run_ms = ms;
  n->last_kernel_ms = kernel_ms;
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaEventDestroy(k0);
  cudaEventDestroy(k1);
  return 0;
}

// Device profile of the step kernel: per instance and phase, SM clock cycles
// summed over the instance's CTAs and steps (phases: 0 update/threshold/reset,
// 1 barrier after it, 2 spike lists and monitors, 3.. one per pathway, last the
// barrier after propagation).  The reference's analogue is run(profile=True)
// (templates/common_group.cpp:72-90).
int b200_set_profiling(b200_net* n, int32_t enable) {
  if (!n) return B200_ERR_ARG;
  n->profiling = enable != 0;
  n->graph_steps = -1;
  if (n->profiling) {
    int r = b200_alloc(n, n->prof, (size_t)n->n_inst * n->M->n_phases * 8);
    if (r) return r;
    B200_CU(n, cudaStreamSynchronize(n->stream));
  }
  return 0;
}

int b200_get_profile(b200_net* n, int32_t inst, uint64_t* cycles, int32_t n_phases) {
  if (!n || inst < 0 || inst >= n->n_inst || n_phases != n->M->n_phases || !n->prof.p) return B200_ERR_ARG;
  B200_CU(n, cudaMemcpy(cycles, (char*)n->prof.p + (size_t)inst * n_phases * 8, (size_t)n_phases * 8,
                        cudaMemcpyDeviceToHost));
  return 0;
}

int b200_profile_phases(b200_net* n, int32_t* count) {
  if (!n || !count) return B200_ERR_ARG;
  *count = n->M->n_phases;
  return 0;
}

// Owner-mode delivery on (default) or off.  In owner mode each CTA of a
// multi-CTA instance owns the target neurons of its tiles: it keeps their
// state in shared memory for the launch, takes every spike of the step from
// the spike lists and delivers only into its own neurons, through per-CTA
// event FIFOs ordered by due step (delays >= 1) or at once (no delay).  It
// applies when every on_pre only adds synaptic values or constants into
// variables of its target (the model library says so).  The reference has one
// delivery path (CSpikeQueue, brian2/synapses/spikequeue.h:14-206); both modes
// reproduce it.
int b200_set_owner(b200_net* n, int32_t enable) {
  if (!n || enable < 0 || enable > 2) return B200_ERR_ARG;
  n->allow_owner = enable;
  n->prepared = false;
  return 0;
}

// Push-mode delivery: 0 off, 1 on where the model allows it, 2 auto (default:
// float32 models with synaptic delays on instances of 2+ CTAs).  In push mode
// each CTA delivers the spikes of the neurons it owns: every delay is at least
// one step, so right after arriving at the barrier of step ts it gathers the
// synapses of its spikes due at step ts+1 and adds their values into an
// accumulator buffer of each delivered variable; after the barrier of step
// ts+1 each owner adds the buffer into its neurons' state.  One barrier per
// step and no global spike list; the order of the additions into a variable
// is the only change against the reference's CSpikeQueue delivery
// (brian2/synapses/spikequeue.h:14-206, templates/synapses.cpp:20-49).
int b200_set_push(b200_net* n, int32_t enable) {
  if (!n || enable < 0 || enable > 2) return B200_ERR_ARG;
  n->allow_push = enable;
  n->prepared = false;
  return 0;
}

// 1 if the current launch plan uses push-mode delivery.
int b200_push_active(b200_net* n, int32_t* active) {
  if (!n || !active) return B200_ERR_ARG;
  int r;
  if (!n->prepared && (r = b200_prepare(n))) return r;
  *active = n->push;
  return 0;
}

// 1 if the current launch plan uses owner-mode delivery.
int b200_owner_active(b200_net* n, int32_t* active) {
  if (!n || !active) return B200_ERR_ARG;
  int r;
  if (!n->prepared && (r = b200_prepare(n))) return r;
  *active = n->owner;
  return 0;
}

// Owner-mode event FIFO size per CTA, in units of the CTA's incoming synapses
// (default 1: every synapse may carry one event in flight).
int b200_set_event_capacity(b200_net* n, double factor) {
  if (!n || !(factor > 0.0)) return B200_ERR_ARG;
  n->ev_factor = factor;
  n->prepared = false;
  return 0;
}

// Spikes of a spike generator group (SpikeGeneratorGroup,
// brian2/input/spikegeneratorgroup.py:21; emission as
// brian2/devices/cpp_standalone/templates/spikegenerator.cpp:5-31): the time
// bin and neuron of every spike, sorted by time bin; `period_bins` > 0 repeats
// them with that period; `last` is the first spike still to emit.
int b200_set_generator(b200_net* n, int32_t inst, int32_t group, const int32_t* bins, const int32_t* index,
                       int64_t count, int32_t period_bins, int32_t last) {
  if (!n || inst < 0 || inst >= n->n_inst || group < 0 || group >= n->M->n_groups || count < 0 ||
      !n->M->groups[group].generator || count > INT32_MAX || last < 0 || last > count ||
      (count && (!bins || !index)))
    return b200_fail(n, B200_ERR_ARG, "bad generator group or arguments");
  b200_group_h& G = n->inst[inst].g[group];
  for (int64_t k = 0; k < count; ++k) {
    if (index[k] < 0 || index[k] >= G.N) return b200_fail(n, B200_ERR_INDEX, "generator spike %lld: neuron out of range", (long long)k);
    if (k && bins[k] < bins[k - 1]) return b200_fail(n, B200_ERR_ARG, "generator spikes not sorted by time bin");
  }
  int r;
  if ((r = b200_alloc(n, G.gen_bins, (size_t)std::max<int64_t>(count, 1) * 4, false))) return r;
  if ((r = b200_alloc(n, G.gen_index, (size_t)std::max<int64_t>(count, 1) * 4, false))) return r;
  if ((r = b200_alloc(n, G.gen_last, 16))) return r;
  if (count) {
    B200_CU(n, cudaMemcpyAsync(G.gen_bins.p, bins, (size_t)count * 4, cudaMemcpyHostToDevice, n->stream));
    B200_CU(n, cudaMemcpyAsync(G.gen_index.p, index, (size_t)count * 4, cudaMemcpyHostToDevice, n->stream));
  }
  B200_CU(n, cudaMemcpyAsync(G.gen_last.p, &last, 4, cudaMemcpyHostToDevice, n->stream));
  B200_CU(n, cudaStreamSynchronize(n->stream));
  G.gen_n = count;
  G.gen_period = std::max(period_bins, 0);
  n->prepared = false;
  return 0;
}

// The random generator of the step loop (the reference's MT19937 state as the
// C++ library stores it: 624 words and the position), continuing at the
// current step.  Replaces the standalone program's brian::_random_generators[0]
// (brian2/devices/cpp_standalone/templates/objects.cpp:426-453).
int b200_set_rng(b200_net* n, int32_t inst, const uint32_t* words, int32_t position) {
  if (!n || inst < 0 || inst >= n->n_inst || !words || position < 0 || position > 624)
    return b200_fail(n, B200_ERR_ARG, "bad generator state");
  b200_inst_h& I = n->inst[inst];
  int r;
  if ((r = b200_alloc(n, I.rng_state, 625 * 4, false))) return r;
  if ((r = b200_alloc(n, I.rng_gauss, 16, false))) return r;
  std::vector<uint32_t> st(words, words + 624);
  st.push_back((uint32_t)position);
  B200_CU(n, cudaMemcpy(I.rng_state.p, st.data(), 625 * 4, cudaMemcpyHostToDevice));
  const double g[2] = {0.0, 0.0};  // no value kept by randn()
  B200_CU(n, cudaMemcpy(I.rng_gauss.p, g, 16, cudaMemcpyHostToDevice));
  I.rng_from = I.rng_to = I.ts;
  I.rng_set = true;
  return 0;
}

// randn()'s kept value (the second value of its last pair, returned by the
// next call; RandomGenerator::randn, objects.cpp:455-477).
int b200_set_rng_gauss(b200_net* n, int32_t inst, int32_t has, double value) {
  if (!n || inst < 0 || inst >= n->n_inst || !n->inst[inst].rng_set)
    return b200_fail(n, B200_ERR_ARG, "set the generator (b200_set_rng) first");
  b200_inst_h& I = n->inst[inst];
  if (I.rng_to != I.ts) return b200_fail(n, B200_ERR_ARG, "the generator has draws ahead of the step");
  const double g[2] = {has ? 1.0 : 0.0, value};
  B200_CU(n, cudaMemcpy(I.rng_gauss.p, g, 16, cudaMemcpyHostToDevice));
  return 0;
}
int b200_get_rng_gauss(b200_net* n, int32_t inst, int32_t* has, double* value) {
  if (!n || inst < 0 || inst >= n->n_inst || !n->inst[inst].rng_set) return b200_fail(n, B200_ERR_ARG, "no generator");
  double g[2];
  B200_CU(n, cudaMemcpy(g, n->inst[inst].rng_gauss.p, 16, cudaMemcpyDeviceToHost));
  if (has) *has = g[0] != 0.0;
  if (value) *value = g[1];
  return 0;
}

// The generator's state after the draws made so far (draws the step loop has
// not consumed yet are included: `unused` reports how many steps of them).
int b200_get_rng(b200_net* n, int32_t inst, uint32_t* words, int32_t* position, int64_t* unused_steps) {
  if (!n || inst < 0 || inst >= n->n_inst || !n->inst[inst].rng_set) return b200_fail(n, B200_ERR_ARG, "no generator");
  std::vector<uint32_t> st(625);
  B200_CU(n, cudaMemcpy(st.data(), n->inst[inst].rng_state.p, 625 * 4, cudaMemcpyDeviceToHost));
  if (words) memcpy(words, st.data(), 624 * 4);
  if (position) *position = (int32_t)st[624];
  if (unused_steps) *unused_steps = n->inst[inst].rng_to - n->inst[inst].ts;
  return 0;
}

// The generator's cursor after a run (the `_lastindex` the reference keeps).
int b200_get_generator(b200_net* n, int32_t inst, int32_t group, int32_t* last) {
  if (!n || inst < 0 || inst >= n->n_inst || group < 0 || group >= n->M->n_groups || !last ||
      !n->M->groups[group].generator || !n->inst[inst].g[group].gen_last.p)
    return b200_fail(n, B200_ERR_ARG, "bad generator group");
  B200_CU(n, cudaMemcpy(last, n->inst[inst].g[group].gen_last.p, 4, cudaMemcpyDeviceToHost));
  return 0;
}

// Thread-block clusters for instances of 2..16 CTAs (hardware barrier) on
// (default) or off (bounded atomic barrier, cooperative launch).
int b200_set_clusters(b200_net* n, int32_t enable) {
  if (!n) return B200_ERR_ARG;
  n->use_clusters = enable != 0;
  n->prepared = false;
  return 0;
}

int b200_launch_plan(b200_net* n, int32_t* grid, int32_t* cluster, int32_t* state_bytes) {
  if (!n) return B200_ERR_ARG;
  int r;
  if (!n->prepared && (r = b200_prepare(n))) return r;
  if (grid) *grid = n->grid;
  if (cluster) *cluster = n->cluster;
  if (state_bytes) *state_bytes = n->state_bytes;
  return 0;
}

// Shared-memory state cache (single-CTA instances: all used variables;
// multi-CTA classic instances: each CTA's own neurons' private variables) on
// (default) or off.
int b200_set_smem_cache(b200_net* n, int32_t enable) {
  if (!n) return B200_ERR_ARG;
  n->smem_cache = enable != 0;
  n->prepared = false;
  return 0;
}

// Test hook: bounded-wait limit, and a CTA rank that leaves before its first
// barrier of the next launch (so the instance barrier must time out).
int b200_set_wait_limit(b200_net* n, int64_t limit_ns, int32_t fault_rank) {
  if (!n || limit_ns <= 0) return B200_ERR_ARG;
  n->limit_ns = (uint64_t)limit_ns;
  n->fault_rank = fault_rank;
  if (fault_rank >= 0) n->prepared = false;  // the fault hook needs the bounded barrier
  return 0;
}

int b200_get_step(b200_net* n, int32_t inst, int64_t* ts) {
  if (!n || inst < 0 || inst >= n->n_inst || !ts) return B200_ERR_ARG;
  *ts = n->inst[inst].ts;
  return 0;
}

int b200_set_step(b200_net* n, int32_t inst, int64_t ts) {
  if (!n || inst < 0 || inst >= n->n_inst || ts < 0) return B200_ERR_ARG;
  n->inst[inst].ts = ts;
  n->inst[inst].stale = false;
  n->inst[inst].rng_from = n->inst[inst].rng_to = ts;  // (the random stream continues from the generator)
  return 0;
}

int b200_last_run_ms(b200_net* n, double* ms) {
  if (!n || !ms) return B200_ERR_ARG;
  *ms = n->last_run_ms;
  return 0;
}

int b200_last_kernel_ms(b200_net* n, double* ms) {
  if (!n || !ms) return B200_ERR_ARG;
  *ms = n->last_kernel_ms;
  return 0;
}

int b200_spikemon_size(b200_net* n, int32_t inst, int32_t mon, int64_t* count) {
  if (!n || inst < 0 || inst >= n->n_inst || mon < 0 || mon >= n->M->n_spkmon || !count) return B200_ERR_ARG;
  b200_spkmon_h& S = n->inst[inst].sm[mon];
  *count = 0;
  if (!S.n.p) return 0;
  B200_CU(n, cudaMemcpy(count, S.n.p, 8, cudaMemcpyDeviceToHost));
  return 0;
}

// i, ts: [count] (count from b200_spikemon_size); per_neuron: [hi-lo] or NULL
int b200_spikemon_get(b200_net* n, int32_t inst, int32_t mon, int32_t* i, int32_t* ts,
                      int32_t* per_neuron, int64_t count) {
  int64_t have = 0;
  int r = b200_spikemon_size(n, inst, mon, &have);
  if (r) return r;
  if (count != have) return b200_fail(n, B200_ERR_ARG, "spike monitor size mismatch");
  b200_spkmon_h& S = n->inst[inst].sm[mon];
  if (count) {
    if (i) B200_CU(n, cudaMemcpy(i, S.i.p, (size_t)count * 4, cudaMemcpyDeviceToHost));
    if (ts) B200_CU(n, cudaMemcpy(ts, S.ts.p, (size_t)count * 4, cudaMemcpyDeviceToHost));
  }
  if (per_neuron && S.count.p && S.hi > S.lo)
    B200_CU(n, cudaMemcpy(per_neuron, S.count.p, (size_t)(S.hi - S.lo) * 4, cudaMemcpyDeviceToHost));
  return 0;
}

int b200_spikemon_values(b200_net* n, int32_t inst, int32_t mon, double* vals, int64_t count) {
  int64_t have = 0;
  int r = b200_spikemon_size(n, inst, mon, &have);
  if (r) return r;
  if (count != have) return b200_fail(n, B200_ERR_ARG, "spike monitor size mismatch");
  const int nv = n->M->spkmon[mon].n_vars;
  if (nv == 0 || count == 0) return 0;
  if (!vals) return B200_ERR_ARG;
  B200_CU(n, cudaMemcpy(vals, n->inst[inst].sm[mon].vals.p, (size_t)count * nv * 8, cudaMemcpyDeviceToHost));
  return 0;
}

int b200_ratemon_size(b200_net* n, int32_t inst, int32_t mon, int64_t* steps) {
  if (!n || inst < 0 || inst >= n->n_inst || mon < 0 || mon >= n->M->n_ratemon || !steps) return B200_ERR_ARG;
  *steps = n->inst[inst].ts - n->inst[inst].rm[mon].step0;
  return 0;
}

// counts: [steps] spikes per step (rate = count/dt/N is formed by the caller,
// as in brian2/devices/cpp_standalone/templates/ratemonitor.cpp:33)
int b200_ratemon_get(b200_net* n, int32_t inst, int32_t mon, int32_t* counts, int64_t steps) {
  int64_t have = 0;
  int r = b200_ratemon_size(n, inst, mon, &have);
  if (r) return r;
  if (steps != have) return b200_fail(n, B200_ERR_ARG, "rate monitor size mismatch");
  if (steps) B200_CU(n, cudaMemcpy(counts, n->inst[inst].rm[mon].cnt.p, (size_t)steps * 4, cudaMemcpyDeviceToHost));
  return 0;
}

int b200_statemon_size(b200_net* n, int32_t inst, int32_t mon, int64_t* steps) {
  if (!n || inst < 0 || inst >= n->n_inst || mon < 0 || mon >= n->M->n_statemon || !steps) return B200_ERR_ARG;
  b200_statemon_h& S = n->inst[inst].stm[mon];
  *steps = 0;
  if (S.n.p) B200_CU(n, cudaMemcpy(steps, S.n.p, 8, cudaMemcpyDeviceToHost));
  return 0;
}

// data: [steps][n_vars][n_rec] as double
int b200_statemon_get(b200_net* n, int32_t inst, int32_t mon, double* data, int64_t steps) {
  int64_t have = 0;
  int r = b200_statemon_size(n, inst, mon, &have);
  if (r) return r;
  if (steps != have) return b200_fail(n, B200_ERR_ARG, "state monitor size mismatch");
  b200_statemon_h& S = n->inst[inst].stm[mon];
  if (steps) B200_CU(n, cudaMemcpy(data, S.data.p, (size_t)steps * S.n_rec * S.n_vars * 8, cudaMemcpyDeviceToHost));
  return 0;
}

// Clears spike/rate/state monitors of one instance (new recording window).
int b200_reset_monitors(b200_net* n, int32_t inst) {
  if (!n || inst < 0 || inst >= n->n_inst) return B200_ERR_ARG;
  b200_inst_h& I = n->inst[inst];
  for (auto& S : I.sm) {
    if (S.n.p) B200_CU(n, cudaMemset(S.n.p, 0, 8));
    if (S.count.p) B200_CU(n, cudaMemset(S.count.p, 0, S.count.bytes));
  }
  for (auto& S : I.rm) S.step0 = I.ts;
  for (auto& S : I.stm) {
    S.step0 = I.ts;
    if (S.n.p) B200_CU(n, cudaMemset(S.n.p, 0, 8));
  }
  return 0;
}

int b200_model_name(char* buf, int64_t len) {
  if (!buf || len <= 0) return B200_ERR_ARG;
  snprintf(buf, (size_t)len, "%s", B200_MODEL.name);
  return 0;
}

int b200_device_bytes(b200_net* n, int64_t* bytes) {
  if (!n || !bytes) return B200_ERR_ARG;
  *bytes = (int64_t)n->device_bytes;
  return 0;
}

int b200_launch_count(b200_net* n, int64_t* count) {
  if (!n || !count) return B200_ERR_ARG;
  *count = n->launches;
  return 0;
}

}  // extern "C"
