// Device-side building blocks of the b200 step engine (sm_103a).
//
// The generated model file (see brian2_gb300/codegen.py) includes this header
// and emits one persistent step kernel per model.  Everything here is model
// independent: the per-instance descriptor layout shared with the host runtime,
// the bounded instance barrier, order-preserving block compaction, block scans,
// and the device versions of Brian's C++ function table
// (brian2/codegen/generators/cpp_generator.py:567-618).
#pragma once
#include <cstdint>
#include <cmath>
#include <cuda_runtime.h>

#define B200_MAX_GROUPS 4
#define B200_MAX_PATHWAYS 8
#define B200_MAX_VARS 24
#define B200_MAX_SPKMON 4
#define B200_MAX_RATEMON 4
#define B200_MAX_STATEMON 4
#define B200_MAX_SUMMED 4
#define B200_MAX_DRAWS 8
#define B200_MAX_THREADS 1024
#define B200_MAX_WARPS (B200_MAX_THREADS / 32)

// status codes written by kernels (mirrored in include/b200.h)
#define B200_OK 0
#define B200_ERR_BARRIER_TIMEOUT 4
#define B200_ERR_INDEX 5
#define B200_ERR_EVENT_OVERFLOW 6
#define B200_ERR_RANDOM 7         // a binomial draw needed a second random number
#define B200_MAX_PAYLOAD 4
#define B200_OWNER_RING 4   // spike-list slots in owner mode (see the kernel's ordering argument)
#define B200_MAX_ACC 8      // push mode: neuron variables that receive deliveries
#define B200_PUSH_BUFS 3    // push mode: accumulator buffers per variable (deliveries of 3 steps)

// ---------------------------------------------------------------------------
// Descriptors (plain data, filled by the host runtime, read by the kernel).
// ---------------------------------------------------------------------------
struct b200_group_d {
  int32_t N;              // neurons of this group in this instance
  int32_t R;              // spike-ring slots (max outgoing delay + 1)
  int32_t n_tiles;        // tiles of this group (each owned by one CTA)
  int32_t own_off;        // >= 0: byte offset in shared memory of this CTA's copy of its own
                          // spike lists (own_cap entries) and tile counts (own_tiles entries)
  int32_t own_cap, own_tiles;
  const int32_t* tile_start;     // [n_tiles+1] first neuron of each tile
  const int32_t* cta_tile;       // [n_cta+1]  first tile of each CTA of the instance
  int32_t* scratch;       // [N]       this step's spikes at tile_start[u]+j
  int32_t* tile_cnt;      // [n_tiles] this step's spike count per tile
  int32_t* ring;          // [R*N]     spikes of step ts at ring[(ts%R)*N ...] (ascending)
  int32_t* ring_total;    // [R]       number of spikes stored in each slot
  int32_t* ring_prefix;   // [R*(n_tiles+1)] per-slot prefix of tile counts
  void* var[B200_MAX_VARS];      // state variables (SoA, length N)
  const double* S;        // scalar table (update | threshold | reset)
  // spike generator groups (SpikeGeneratorGroup): spikes from sorted lists
  const int32_t* gen_bins;   // [gen_n] time bin of each spike (non-decreasing)
  const int32_t* gen_index;  // [gen_n] neuron of each spike
  int64_t gen_n;
  int32_t* gen_last;         // [1] next spike to emit (persists across launches)
  int32_t gen_period;        // period in steps (0: no repetition)
  // push mode: each CTA's spike list of the last RH steps, compact and ascending,
  // at hist[(ts % RH) * N + first own neuron + k]; the first HCAP entries of each
  // slot also in shared memory at byte offset hist_off, the slot counts at hcnt_off
  int32_t RH, HCAP;
  int32_t hist_off, hcnt_off;
  int32_t* hist;             // [RH * N]
  int32_t* hcnt;             // [RH * n_cta] spikes of each CTA per slot
};

// Owner mode: per (pathway, CTA) FIFO of delivery events.  Every step the CTA
// appends one *batch* (the events of that step's spikes, sorted by delay) at
// `head`; a batch is retired once its largest delay is due, so the records
// form a circular FIFO of `cap` (a power of two) entries.  Arrays are per CTA:
// element [rank * cap + i], state [rank * 2 + {0: head, 1: tail}], batch
// table [rank * RB + b] (absolute base, step tag) and [rank * RB + b][W + 1]
// (exclusive per-delay offsets within the batch).
struct b200_fifo_d {
  int64_t cap;            // records per CTA (power of two)
  int32_t RB, W;          // batch-table slots, delays per batch
  int32_t tab_off, _pad;  // byte offset of this CTA's batch table in shared memory (when cached there)
  int32_t* tgt;           // [n_cta * cap] target neuron (within the target group)
  void* pay[B200_MAX_PAYLOAD];  // [n_cta * cap] payload values (synaptic variables)
  int64_t* state;         // [n_cta * 2] head, tail (absolute record positions)
  int64_t* base;          // [n_cta * RB] first record of each batch
  int64_t* tag;           // [n_cta * RB] step of the spikes of each batch (-1: none)
  int32_t* off;           // [n_cta * RB * (W + 1)] per-delay offsets in each batch
};

struct b200_pathway_d {
  int32_t D;              // largest delay in steps (0 = no delays)
  int32_t src_lo, src_hi; // presynaptic neuron range within the source group
  int32_t tile_lo, tile_hi;  // source-group tiles covering [src_lo, src_hi)
  int32_t dmin;           // smallest delay in steps
  int64_t n_syn;
  const int64_t* segptr;  // [(src_hi-src_lo)*(D+1)+1] CSR over (source, delay slot)
  const int32_t* post;    // [n_syn] target neuron (within target group), CSR order
  const int32_t* pre;     // [n_syn] source neuron (within source group), CSR order
  void* var[B200_MAX_VARS];  // synaptic variables in CSR order (owner mode: owner order)
  const double* S;        // scalar table of on_pre
  const int64_t* sidx;    // shared synapses: [n_syn] the synapse's position in the owning
                          // pathway's order (post/pre/var then point to that pathway's arrays)
  // owner mode: segptr is over (source, owning CTA) with n_cta entries per
  // source, post/var are in that order, odelay is each synapse's delay slot
  const uint16_t* odelay;
  b200_fifo_d ev;
  // push mode: byte offset in shared memory of the per-slot bounds (int2, RH of the
  // source group) of the CTA's spikes in [src_lo, src_hi)
  int32_t pb_off, _pad_p;
};

struct b200_spkmon_d {
  int32_t group, lo, hi, tile_lo, tile_hi, n_vars;
  int64_t cap;            // capacity of i/ts
  int64_t* n;             // [1] number of recorded spikes
  int32_t* i;             // [cap] neuron index - lo
  int32_t* ts;            // [cap] time step of the spike
  int32_t* count;         // [hi-lo] spikes per neuron
  // recorded variables (SpikeMonitor(..., variables=...)): their values when the
  // step's thresholder ran, as double
  double* snap;           // [n_vars][group N] the values of the step's spiking neurons
  double* vals;           // [cap][n_vars] one row per recorded spike
  int32_t* xcnt;          // push mode: [3][n_cta] each CTA's recorded spikes of a step (by step % 3)
};

struct b200_ratemon_d {
  int32_t group, lo, hi, tile_lo, tile_hi, _pad;
  int64_t step0;          // time step of cnt[0]
  int64_t cap;            // steps available in cnt
  int32_t* cnt;           // [cap] spikes in [lo,hi) per step
  int32_t* xcnt;          // push mode: [3][n_cta] each CTA's spikes in [lo,hi) of a step (by step % 3)
};

struct b200_statemon_d {
  int32_t group, n_rec, n_vars, _pad;
  const int32_t* idx;     // [n_rec] recorded neuron indices
  int32_t var_id[8];      // which state variables
  int32_t var_dbl[8];     // 1 if the variable is double, 0 if float
  int64_t step0, cap;     // recording starts at step0; rows available
  int64_t* n;             // [1] number of recorded rows
  double* data;           // [cap][n_vars][n_rec] values (as double), one row per recorded step
};

// A summed variable (SummedVariableUpdater, brian2/synapses/synapses.py:116-175;
// templates/summed_variable.cpp): each target neuron's value is the sum, in
// synapse creation order, of an expression over its synapses.
struct b200_summed_d {
  int32_t lo, hi;         // target neurons [lo, hi) of the target group
  const int64_t* seg;     // [hi-lo+1] each target's run in syn
  const int64_t* syn;     // the synapses' positions in their pathway's arrays, creation order per target
};

struct b200_inst_d {
  int32_t cta0, n_cta;    // CTAs [cta0, cta0+n_cta) of the grid run this instance
  int32_t cache_bytes;    // >0: single-CTA instance whose state is cached in shared memory
  int32_t cache_lists;    // 1: the step's spike list and tile counts are cached too
  int64_t ts;             // next time step to execute
  int64_t ts_end;         // stop before this step
  double dt;
  unsigned int* bar;      // [2] barrier arrival counter, generation
  int32_t* status;        // [1] error status of this instance
  int64_t* ts_done;       // [1] written at exit: first step not executed
  int32_t* pending_reset; // [B200_MAX_GROUPS] reset of the last step still to apply
  // owner mode (b200_owner_kernel): each CTA delivers into the neurons it owns
  int32_t owner;          // 1: this instance runs in owner mode
  int32_t lag;            // 1: every delay >= 1 step (owner: a step pushes the previous step's spikes;
                          // classic: deliveries are prepared while barrier A completes)
  int64_t ts_base;        // step whose arrival count starts at 0 in bar64
  unsigned long long* bar64;  // [1] arrivals of the split barrier
  int32_t tab_smem;       // 1: the batch tables are kept in shared memory for the launch
  int32_t stage_off;      // byte offset of the event staging area in shared memory
  int32_t stage_cap;      // events it holds (0: none; pushes take two passes over global memory)
  int32_t priv_bytes;     // classic multi-CTA instance: bytes of each CTA's shared-memory copy of
                          // its own neurons' private variables (0: none)
  // push mode (b200_push_kernel): each CTA delivers its own neurons' spikes, one step
  // ahead, into accumulators that the target's owner adds to its state after the
  // step's barrier; acc[k] is [B200_PUSH_BUFS][N] of the model's k-th delivered variable
  int32_t push, _pad_push;
  void* acc[B200_MAX_ACC];
  b200_group_d g[B200_MAX_GROUPS];
  b200_pathway_d p[B200_MAX_PATHWAYS];
  b200_spkmon_d sm[B200_MAX_SPKMON];
  b200_ratemon_d rm[B200_MAX_RATEMON];
  b200_statemon_d stm[B200_MAX_STATEMON];
  b200_summed_d sum[B200_MAX_SUMMED];
  // random numbers of the step loop: the reference's stream, drawn ahead of the
  // launch in its order by b200_variates_kernel, one double per draw
  const double* rng_vals;     // [steps of the launch][rng_per_step], from step rng_ts0
  int64_t rng_ts0;            // step of rng_vals[0]
  int32_t rng_per_step;       // draws per step (all draw sites)
  int32_t draw_off[B200_MAX_DRAWS];  // first draw of each site within a step
  int32_t _pad_r;
};

static_assert(sizeof(b200_inst_d) % 8 == 0, "descriptor is copied in 8-byte words");

// ---------------------------------------------------------------------------
// Model tables: emitted by the code generator, read by the host runtime.
// ---------------------------------------------------------------------------
enum b200_kind { B200_F64 = 0, B200_F32 = 1, B200_I32 = 2, B200_I8 = 3, B200_I64 = 4 };
static inline size_t b200_kind_size(int k) {
  switch (k) {
    case B200_F64: return 8;
    case B200_F32: return 4;
    case B200_I32: return 4;
    case B200_I8: return 1;
    case B200_I64: return 8;
  }
  return 0;
}

struct b200_group_info {
  const char* name;
  int n_vars;
  const char* const* var_names;
  const int* var_kind;
  int n_scalars;  // size of the scalar table
  const int* var_used;  // 1 if the step code touches the variable
  int generator;  // 1: a spike generator group (spikes from b200_set_generator lists)
  const int* var_private;  // 1: used, and touched only by the CTA that owns the neuron (no
                           // pathway or other group reads or writes it)
  int alias;  // a custom event's group: the group whose state it shares (its events' lists
              // are this group's spike lists); -1 otherwise
};
struct b200_pathway_info {
  const char* name;
  int src_group, tgt_group;
  int n_vars;
  const char* const* var_names;
  const int* var_kind;
  int n_scalars;
  // owner mode: the synaptic variables on_pre reads (carried by each event)
  int n_payload;
  const int* payload_var;
  // >= 0: this pathway (the on_post pathway of a Synapses object) shares the
  // synapses and synaptic variables of that pathway (its on_pre pathway)
  int alias;
};
// A draw site: a code object of the step loop that draws from the reference's
// generator, `calls` draws per neuron of [lo, hi) of a group (hi < 0: to the
// group's end) and step -- rand() in threshold code (PoissonGroup), randn() in
// a state update (stochastic equations), the binomial counts of a PoissonInput
// (brian2/input/poissoninput.py:20-141, brian2/input/binomial.py:93-141).
struct b200_draw_info {
  const char* name;
  int kind;                   // B200_DRAW_*
  int group, lo, hi, calls;
  int n, reverse;             // binomial: trials, sampler counts failures
  double qn, bound, p, q;     // binomial by inversion (the reference's printed constants)
  double scale, loc;          // binomial, normal approximation
};
struct b200_summed_info {
  const char* name;
  int pathway;     // the pathway holding the Synapses object's synapses and variables
  int tgt_group;   // group of the summed variable
  int tgt_var;     // its index among the group's variables
  int index_post;  // 1: summed into the postsynaptic neuron, 0: into the presynaptic one
};
struct b200_mon_info {
  const char* name;
  int group;
  int every;   // records on every k-th step (a state monitor on a slower clock); 1 otherwise
  int n_vars;  // a spike monitor's recorded variables besides i and t
  int syn;     // a state monitor of a Synapses object: the pathway holding its synapses; -1 otherwise
};
struct b200_model_info {
  const char* name;
  int n_groups, n_pathways, n_spkmon, n_ratemon, n_statemon;
  const b200_group_info* groups;
  const b200_pathway_info* pathways;
  const b200_mon_info* spkmon;
  const b200_mon_info* ratemon;
  const b200_mon_info* statemon;
  int n_consts;
  const char* const* const_names;
  const double* const_defaults;
  // evaluates the scalar table of a group (kind 0) or pathway (kind 1)
  void (*eval_scalars)(int kind, int id, const double* consts, double dt, double* out);
  // launches the step kernel
  cudaError_t (*launch)(b200_inst_d* insts, const int2* cta_map, int n_inst, int queue_mode,
                        int* work, int64_t max_steps, uint64_t limit_ns, int grid, int threads,
                        int cooperative, int max_tiles1, int max_w, int fault_rank, int state_bytes,
                        unsigned long long* prof, int cluster, cudaStream_t s);
  int (*max_active_ctas)(int threads, int max_tiles1, int max_w, int state_bytes);
  int (*static_smem)(int threads);
  int (*max_cluster)(int threads, int max_tiles1, int max_w, int state_bytes, int cluster);
  int n_phases;  // device profile: A, barrier A, spike lists, one per pathway, barrier B
  // 1: every pathway's on_pre only adds to variables of its target neuron from
  // synaptic values and constants, so owner-mode delivery applies
  int owner_ok;
  int owner_event_bytes;  // shared-memory bytes per staged event
  int n_summed;
  const b200_summed_info* summed;
  // the code objects that draw random numbers, in the order the reference's
  // schedule runs them in a step (the order of the draws)
  int n_draws;
  const b200_draw_info* draws;
  // 1: push-mode delivery applies (owner_ok, and no spike generator or custom event
  // is the source of a pathway); the delivered variables as (group, variable) pairs
  int push_ok;
  int n_acc;
  const int* acc_vars;  // [2 * n_acc]
};
// `tcode` bit selecting the owner-mode kernel
#define B200_TCODE_OWNER (1 << 20)
// `tcode` bit selecting the push-mode kernel
#define B200_TCODE_PUSH (1 << 21)


// ---------------------------------------------------------------------------
// Small utilities
// ---------------------------------------------------------------------------
__device__ __forceinline__ unsigned b200_lanemask_lt() {
  unsigned m;
  asm("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
  return m;
}

__device__ __forceinline__ unsigned b200_ld_acquire(const unsigned* p) {
  unsigned v;
  asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}

__device__ __forceinline__ void b200_st_release(unsigned* p, unsigned v) {
  asm volatile("st.release.gpu.global.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}

__device__ __forceinline__ unsigned long long b200_ld_acquire64(const unsigned long long* p) {
  unsigned long long v;
  asm volatile("ld.acquire.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
  return v;
}

__device__ __forceinline__ void b200_red_release_add64(unsigned long long* p, unsigned long long v) {
  asm volatile("red.release.gpu.global.add.u64 [%0], %1;" ::"l"(p), "l"(v) : "memory");
}

__device__ __forceinline__ void b200_red_relaxed_add64(unsigned long long* p, unsigned long long v) {
  asm volatile("red.relaxed.gpu.global.add.u64 [%0], %1;" ::"l"(p), "l"(v) : "memory");
}

__device__ __forceinline__ uint64_t b200_globaltimer() {
  uint64_t t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

// Exclusive block-wide scan of one int per thread.  `wsum` is smem of
// B200_MAX_WARPS+1 ints.  Returns the exclusive prefix; *total gets the sum.
// All threads of the block must call it.
__device__ __forceinline__ int b200_block_exscan(int x, int* wsum, int* total) {
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const int nw = (blockDim.x + 31) >> 5;
  int v = x;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    int y = __shfl_up_sync(0xffffffffu, v, o);
    if (lane >= o) v += y;
  }
  if (lane == 31) wsum[w] = v;
  __syncthreads();
  if (w == 0) {
    int s = lane < nw ? wsum[lane] : 0;
    int incl = s;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      int y = __shfl_up_sync(0xffffffffu, incl, o);
      if (lane >= o) incl += y;
    }
    if (lane < nw) wsum[lane] = incl - s;
    if (lane == 31) wsum[B200_MAX_WARPS] = incl;
  }
  __syncthreads();
  const int r = wsum[w] + v - x;
  *total = wsum[B200_MAX_WARPS];
  __syncthreads();
  return r;
}

// Order-preserving compaction of one flag per thread (warp ballot + scan of the
// warp counts).  Returns this thread's rank among the set flags of the block in
// thread order; *total gets the number of set flags.
__device__ __forceinline__ int b200_block_compact(bool flag, int* wsum, int* total) {
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const int nw = (blockDim.x + 31) >> 5;
  const unsigned m = __ballot_sync(0xffffffffu, flag);
  if (lane == 0) wsum[w] = __popc(m);
  __syncthreads();
  if (w == 0) {
    int s = lane < nw ? wsum[lane] : 0;
    int incl = s;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      int y = __shfl_up_sync(0xffffffffu, incl, o);
      if (lane >= o) incl += y;
    }
    if (lane < nw) wsum[lane] = incl - s;
    if (lane == 31) wsum[B200_MAX_WARPS] = incl;
  }
  __syncthreads();
  const int r = wsum[w] + __popc(m & b200_lanemask_lt());
  *total = wsum[B200_MAX_WARPS];
  __syncthreads();
  return r;
}

// Block-cooperative copy of `bytes`: 4-byte words when both ends are 4-byte
// aligned, single bytes otherwise (a 1-byte variable from a tile boundary).
__device__ __forceinline__ void b200_prefetch_l2(const void* p) {
  asm volatile("prefetch.global.L2 [%0];" :: "l"(p));
}

__device__ __forceinline__ void b200_copy_bytes(void* dst, const void* src, size_t bytes) {
  if ((((uintptr_t)dst) | ((uintptr_t)src)) & 3) {
    unsigned char* db = (unsigned char*)dst;
    const unsigned char* sb = (const unsigned char*)src;
    for (size_t k = threadIdx.x; k < bytes; k += blockDim.x) db[k] = sb[k];
    return;
  }
  const size_t nw = bytes / 4;
  uint32_t* d = (uint32_t*)dst;
  const uint32_t* s = (const uint32_t*)src;
  for (size_t k = threadIdx.x; k < nw; k += blockDim.x) d[k] = s[k];
  unsigned char* db = (unsigned char*)dst;
  const unsigned char* sb = (const unsigned char*)src;
  for (size_t k = nw * 4 + threadIdx.x; k < bytes; k += blockDim.x) db[k] = sb[k];
}

// Hardware barrier over the CTAs of a thread-block cluster (one instance per
// cluster).  Release/acquire at cluster scope also orders the global-memory
// accesses made before it.  Every CTA of the cluster executes the same
// sequence of these barriers (the step loop's control flow is uniform).
__device__ __forceinline__ void b200_cluster_sync() {
  asm volatile(
      "barrier.cluster.arrive.release.aligned;\n"
      "barrier.cluster.wait.acquire.aligned;\n" ::: "memory");
}

// Barrier over the n_cta CTAs of one instance.  Bounded: after `limit_ns` of
// waiting the instance status is set to B200_ERR_BARRIER_TIMEOUT and the call
// returns false, so a kernel never spins forever.  With n_cta == 1 it is a
// plain __syncthreads.  `gen` counts the barriers this CTA has passed; `rank`
// is the CTA's rank within the instance.
__device__ __forceinline__ bool b200_inst_barrier(const b200_inst_d& I, unsigned& gen,
                                                  uint64_t limit_ns, int cluster, int rank) {
  if (cluster) {
    b200_cluster_sync();
    return true;
  }
  __syncthreads();
  if (I.n_cta == 1) return true;
  __shared__ int ok;
  if (threadIdx.x == 0) {
    // one arrival word, no reset: rank 0 adds 2^31 - (n_cta - 1), every other
    // CTA adds 1, so bit 31 flips exactly when the last CTA has arrived (the
    // scheme of the cooperative-groups grid barrier); waiters poll that bit
    ok = 1;
    const unsigned nb = rank == 0 ? 0x80000000u - (unsigned)(I.n_cta - 1) : 1u;
    __threadfence();
    const unsigned old = atomicAdd(&I.bar[0], nb);
    if (((old + nb) ^ old) & 0x80000000u) {
      __threadfence();  // this CTA completed the barrier: order its reads after the others' writes
    } else {
      const uint64_t t0 = b200_globaltimer();
      int spins = 0;
      while (((b200_ld_acquire(&I.bar[0]) ^ old) & 0x80000000u) == 0) {
        if (++spins > 32) __nanosleep(32);
        if ((spins & 255) == 0 &&
            (b200_globaltimer() - t0 > limit_ns || *((volatile int32_t*)I.status) != 0)) {
          atomicCAS(I.status, 0, B200_ERR_BARRIER_TIMEOUT);
          ok = 0;
          break;
        }
      }
    }
    ++gen;
  }
  __syncthreads();
  return ok != 0;
}

// The same barrier in two halves, so that a CTA can do work that does not
// depend on the other CTAs between its arrival and its wait: b200_inst_arrive
// (all threads; thread 0 keeps the arrival word's old value in `old`), then
// b200_inst_wait (all threads), bounded like b200_inst_barrier.
__device__ __forceinline__ void b200_inst_arrive(const b200_inst_d& I, int cluster, int rank, unsigned& old) {
  if (cluster) {
    asm volatile("barrier.cluster.arrive.release.aligned;\n" ::: "memory");
    return;
  }
  __syncthreads();
  if (I.n_cta == 1) return;
  if (threadIdx.x == 0) {
    const unsigned nb = rank == 0 ? 0x80000000u - (unsigned)(I.n_cta - 1) : 1u;
    __threadfence();
    old = atomicAdd(&I.bar[0], nb);
  }
}

__device__ __forceinline__ bool b200_inst_wait(const b200_inst_d& I, unsigned& gen, uint64_t limit_ns,
                                               int cluster, int rank, unsigned old) {
  if (cluster) {
    asm volatile("barrier.cluster.wait.acquire.aligned;\n" ::: "memory");
    return true;
  }
  if (I.n_cta == 1) {
    __syncthreads();
    return true;
  }
  __shared__ int ok_w;
  if (threadIdx.x == 0) {
    ok_w = 1;
    const unsigned nb = rank == 0 ? 0x80000000u - (unsigned)(I.n_cta - 1) : 1u;
    if (((old + nb) ^ old) & 0x80000000u) {
      __threadfence();  // this CTA completed the barrier
    } else {
      const uint64_t t0 = b200_globaltimer();
      int spins = 0;
      while (((b200_ld_acquire(&I.bar[0]) ^ old) & 0x80000000u) == 0) {
        if (++spins > 32) __nanosleep(32);
        if ((spins & 255) == 0 &&
            (b200_globaltimer() - t0 > limit_ns || *((volatile int32_t*)I.status) != 0)) {
          atomicCAS(I.status, 0, B200_ERR_BARRIER_TIMEOUT);
          ok_w = 0;
          break;
        }
      }
    }
    ++gen;
  }
  __syncthreads();
  return ok_w != 0;
}

// ---------------------------------------------------------------------------
// The reference's random stream (brian2/devices/cpp_standalone/templates/
// objects.cpp:426-478): a 32-bit Mersenne Twister (MT19937, Matsumoto and
// Nishimura 1998); rand() = (a*2^26 + b) / 2^53 from two outputs a = w0 >> 5,
// b = w1 >> 6; randn() by the polar method (Marsaglia), which draws pairs
// until one falls inside the unit circle, returns f*x2 and keeps f*x1 for the
// next call.  How many outputs a step uses depends only on the stream, never on
// the network, so b200_variates_kernel walks the stream ahead of a launch, in
// the reference's order of draws, and writes one double per draw.
// ---------------------------------------------------------------------------
#define B200_MT_N 624
#define B200_MT_M 397
// kinds of draw sites (one per code object that draws, in schedule order)
#define B200_DRAW_UNIFORM 0    // rand()
#define B200_DRAW_NORMAL 1     // randn()
#define B200_DRAW_BINOMIAL 2   // binomial by inversion (brian2/input/binomial.py:93-141)
#define B200_DRAW_BINORMAL 3   // binomial, normal approximation: (float)(randn()*scale + loc)

__device__ __forceinline__ uint32_t b200_mt_mix(uint32_t hi, uint32_t lo, uint32_t far) {
  const uint32_t y = (hi & 0x80000000u) | (lo & 0x7fffffffu);
  return far ^ (y >> 1) ^ ((y & 1u) ? 0x9908b0dfu : 0u);
}
__device__ __forceinline__ uint32_t b200_mt_temper(uint32_t y) {
  y ^= y >> 11;
  y ^= (y << 7) & 0x9d2c5680u;
  y ^= (y << 15) & 0xefc60000u;
  y ^= y >> 18;
  return y;
}
// The next 624 words of the state x (in shared memory), in place.  Sequentially
// x[i] = x[i+M] ^ mix(x[i], x[i+1]) for i = 0..623, indices mod 624: each of
// three sweeps reads the words it needs (x[i+1] before anyone writes it, the far
// word after the previous sweep wrote it), then writes.  All threads of a block
// of at least 624 threads call it.
__device__ __forceinline__ void b200_mt_regen(uint32_t* x) {
  const int t = threadIdx.x;
  uint32_t v = 0;
  if (t < 227) v = b200_mt_mix(x[t], x[t + 1], x[t + B200_MT_M]);
  __syncthreads();
  if (t < 227) x[t] = v;
  __syncthreads();
  if (t >= 227 && t < 454) v = b200_mt_mix(x[t], x[t + 1], x[t - 227]);
  __syncthreads();
  if (t >= 227 && t < 454) x[t] = v;
  __syncthreads();
  if (t >= 454 && t < 623) v = b200_mt_mix(x[t], x[t + 1], x[t - 227]);
  __syncthreads();
  if (t >= 454 && t < 623) x[t] = v;
  __syncthreads();
  if (t == 0) x[623] = b200_mt_mix(x[623], x[0], x[396]);
  __syncthreads();
}
__device__ __forceinline__ double b200_rand2(uint32_t w0, uint32_t w1) {
  const long long a = (long long)(w0 >> 5), b = (long long)(w1 >> 6);
  return ((double)a * 67108864.0 + (double)b) / 9007199254740992.0;
}

// One draw site per step: `count` values (neurons x calls per neuron).
struct b200_site_d {
  int32_t kind, count;
  int32_t n, reverse;           // binomial: trials; 1 = the sampler counts failures
  double qn, bound, p, q;       // binomial by inversion, the reference's printed constants
  double scale, loc;            // normal approximation
};
struct b200_sites_d {
  int32_t n_sites, _pad;
  b200_site_d s[B200_MAX_DRAWS];
};

// The draws of `steps` steps, continuing the generator: state = [624 words,
// position] (the C++ library's form), gauss = [has a kept value (0/1), value]
// (randn()'s cache); out[step][per_step] in site order.  Launch <<<1, 1024>>>.
// A binomial draw past the bound starts over with a new number, as in the
// reference; status gets B200_ERR_RANDOM if that needed more numbers than the
// two blocks of outputs in shared memory hold (never at the probabilities the
// bound allows).
__global__ void __launch_bounds__(1024) b200_variates_kernel(uint32_t* state, double* gauss, b200_sites_d S,
                                                           double* out, int64_t per_step, int64_t steps,
                                                           int32_t* status) {
  __shared__ uint32_t xc[B200_MT_N], xn[B200_MT_N];  // the current and the next block of the state
  __shared__ int s_wsum[B200_MAX_WARPS + 1];
  __shared__ int s_first, s_cend, s_has, s_used;
  __shared__ double s_keep;
  const int t = threadIdx.x;
  if (t < B200_MT_N) { xc[t] = state[t]; xn[t] = state[t]; }
  int p = (int)state[B200_MT_N];  // next output: xc[p] (p == 624: xn[0])
  __syncthreads();
  b200_mt_regen(xn);
  bool has = gauss[0] != 0.0;
  double kept = gauss[1];
  // output o after the read position (o < 1248 - p)
  auto word = [&](int o) -> uint32_t {
    return b200_mt_temper(o < B200_MT_N - p ? xc[p + o] : xn[o - (B200_MT_N - p)]);
  };
  auto advance = [&](int k) {  // all threads, same k
    __syncthreads();
    p += k;
    while (p >= B200_MT_N) {
      if (t < B200_MT_N) xc[t] = xn[t];
      __syncthreads();
      b200_mt_regen(xn);
      p -= B200_MT_N;
    }
  };
  for (int64_t st = 0; st < steps; ++st) {
    double* o_step = out + st * per_step;
    for (int si = 0; si < S.n_sites; ++si) {
      const b200_site_d& D = S.s[si];
      double* const o = o_step;
      o_step += D.count;
      const int64_t K = D.count;
      if (D.kind == B200_DRAW_UNIFORM) {
        for (int64_t i = 0; i < K;) {
          const int C = (int)(K - i < 312 ? K - i : 312);
          if (t < C) o[i + t] = b200_rand2(word(2 * t), word(2 * t + 1));
          advance(2 * C);
          i += C;
        }
      } else if (D.kind == B200_DRAW_NORMAL || D.kind == B200_DRAW_BINORMAL) {
        const bool tr = D.kind == B200_DRAW_BINORMAL;
        auto value = [&](double v) -> double {
          return tr ? (double)__double2float_rn(__dadd_rn(__dmul_rn(v, D.scale), D.loc)) : v;
        };
        int64_t i = 0;
        if (K > 0 && has) {  // the value kept by the previous call
          if (t == 0) o[0] = value(kept);
          has = false;
          i = 1;
        }
        while (i < K) {
          const int64_t need = (K - i + 1) / 2;  // pairs still to accept
          const int C = 156;                     // candidates (4 outputs each) looked at together
          double x1 = 0.0, x2 = 0.0, r2 = 0.0;
          bool acc = false;
          if (t < C) {
            x1 = __dsub_rn(__dmul_rn(2.0, b200_rand2(word(4 * t), word(4 * t + 1))), 1.0);
            x2 = __dsub_rn(__dmul_rn(2.0, b200_rand2(word(4 * t + 2), word(4 * t + 3))), 1.0);
            r2 = __dadd_rn(__dmul_rn(x1, x1), __dmul_rn(x2, x2));
            acc = !(r2 >= 1.0 || r2 == 0.0);
          }
          if (t == 0) { s_cend = C; s_has = 0; }
          int tot;
          const int r = b200_block_compact(acc, s_wsum, &tot);
          const int64_t use = tot < need ? tot : need;
          if (acc && r < use) {
            const double f = __dsqrt_rn(__ddiv_rn(__dmul_rn(-2.0, log(r2)), r2));
            const int64_t j = i + 2 * (int64_t)r;
            o[j] = value(__dmul_rn(f, x2));
            if (j + 1 < K) o[j + 1] = value(__dmul_rn(f, x1));
            else { s_has = 1; s_keep = __dmul_rn(f, x1); }
            if (r == use - 1 && tot >= need) s_cend = t + 1;
          }
          __syncthreads();
          const int used = s_cend;
          if (s_has) { has = true; kept = s_keep; }
          advance(4 * used);
          i += 2 * use;
        }
      } else {  // B200_DRAW_BINOMIAL
        const double nn = (double)D.n;
        for (int64_t i = 0; i < K;) {
          const int C = (int)(K - i < 312 ? K - i : 312);
          if (t == 0) s_first = C;
          __syncthreads();
          if (t < C) {
            double U = b200_rand2(word(2 * t), word(2 * t + 1)), px = D.qn;
            long long X = 0;
            bool redraw = false;
            while (U > px) {
              X++;
              if ((double)X > D.bound) { redraw = true; break; }
              U = __dsub_rn(U, px);
              px = __ddiv_rn(__dmul_rn(__dmul_rn((double)(D.n - X + 1), D.p), px), __dmul_rn((double)X, D.q));
            }
            if (redraw) atomicMin(&s_first, t);
            else o[i + t] = D.reverse ? nn - (double)X : (double)X;
          }
          __syncthreads();
          const int first = s_first;
          if (first == C) {
            advance(2 * C);
            i += C;
            continue;
          }
          // the draws before `first` stand; `first` starts over with new numbers
          advance(2 * first);
          if (t == 0) {
            const int win = 2 * B200_MT_N - p;
            int used = 2;
            double U = b200_rand2(word(0), word(1)), px = D.qn;
            long long X = 0;
            while (U > px) {
              X++;
              if ((double)X > D.bound) {
                X = 0;
                px = D.qn;
                if (used + 2 > win) { atomicCAS(status, 0, B200_ERR_RANDOM); break; }
                U = b200_rand2(word(used), word(used + 1));
                used += 2;
              } else {
                U = __dsub_rn(U, px);
                px = __ddiv_rn(__dmul_rn(__dmul_rn((double)(D.n - X + 1), D.p), px), __dmul_rn((double)X, D.q));
              }
            }
            o[i + first] = D.reverse ? nn - (double)X : (double)X;
            s_used = used;
          }
          __syncthreads();
          advance(s_used);
          i += first + 1;
        }
      }
    }
  }
  __syncthreads();
  if (t < B200_MT_N) state[t] = xc[t];
  if (t == 0) {
    state[B200_MT_N] = (uint32_t)p;
    gauss[0] = has ? 1.0 : 0.0;
    gauss[1] = kept;
  }
}

// ---------------------------------------------------------------------------
// Brian's function table (brian2/codegen/generators/cpp_generator.py:90-197,
// 567-618; brian2/devices/cpp_standalone/brianlib/common_math.h).  Host and
// device: the scalar blocks are evaluated on the host, where the semantics are
// the reference's (double-only _exprel, `pow` resolved through namespace std);
// on the device float arguments stay in float.
// ---------------------------------------------------------------------------
__host__ __device__ __forceinline__ double _exprel(double x) {
  if (fabs(x) < 1e-16) return 1.0;
  if (x > 717) return INFINITY;
  return expm1(x) / x;
}
#ifdef __CUDA_ARCH__
__device__ __forceinline__ float _exprel(float x) {
  if (fabsf(x) < 1e-16f) return 1.0f;
  if (x > 717.0f) return INFINITY;
  return expm1f(x) / x;
}
#else
static inline double _exprel(float x) { return _exprel((double)x); }
#endif
template <typename T>
__host__ __device__ __forceinline__ T _clip(const T value, const double a_min, const double a_max) {
  if (value < a_min) return a_min;
  if (value > a_max) return a_max;
  return value;
}
template <typename T1, typename T2>
__host__ __device__ __forceinline__ auto _brian_pow(T1 a, T2 b) -> decltype(pow(a, b)) {
  using std::pow;
  return pow(a, b);
}
#ifdef __CUDA_ARCH__
// a float base with an integer exponent (Brian writes n**4 as _brian_pow(n, 4)):
// std::pow would promote it to double; on the device a float model stays in
// float (the FP64 pipe runs at a small fraction of the FP32 rate)
__device__ __forceinline__ float _brian_pow(float a, int b) { return powf(a, (float)b); }
__device__ __forceinline__ float _brian_pow(float a, long long b) { return powf(a, (float)b); }
#endif
template <typename T1, typename T2>
__host__ __device__ __forceinline__ double _brian_floordiv(T1 x, T2 y) { return floor(1.0 * x / y); }
__host__ __device__ __forceinline__ int32_t _brian_floordiv(int32_t a, int32_t b) {
  int32_t q = a / b;
  int32_t r = a - q * b;
  q -= ((r != 0) & ((r ^ b) < 0));
  return q;
}
__host__ __device__ __forceinline__ int64_t _brian_floordiv(int64_t a, int64_t b) {
  int64_t q = a / b;
  int64_t r = a - q * b;
  q -= ((r != 0) & ((r ^ b) < 0));
  return q;
}
template <typename T1, typename T2>
__host__ __device__ __forceinline__ double _brian_mod(T1 x, T2 y) { return x - y * floor(1.0 * x / y); }
__host__ __device__ __forceinline__ int32_t _brian_mod(int32_t x, int32_t y) {
  int32_t r = x % y;
  r += ((r != 0) & ((r ^ y) < 0)) * y;
  return r;
}
__host__ __device__ __forceinline__ int64_t _brian_mod(int64_t x, int64_t y) {
  int64_t r = x % y;
  r += ((r != 0) & ((r ^ y) < 0)) * y;
  return r;
}
template <typename T>
__host__ __device__ __forceinline__ int int_(T value) { return (int)value; }
// core/functions.py:771 timestep(t, dt) = int64((t + 1e-3*dt)/dt)
__host__ __device__ __forceinline__ int64_t _timestep(double t, double dt) {
  return (int64_t)((t + 1e-3 * dt) / dt);
}
#define _brian_abs fabs

// Atomic accumulation used by on_pre statements `x_post += expr`.
__device__ __forceinline__ void _b200_atomic_add(double* p, double v) { atomicAdd(p, v); }
__device__ __forceinline__ void _b200_atomic_add(float* p, float v) { atomicAdd(p, v); }
__device__ __forceinline__ void _b200_atomic_add(float* p, double v) { atomicAdd(p, (float)v); }
__device__ __forceinline__ void _b200_atomic_add(int32_t* p, int32_t v) { atomicAdd(p, v); }

// ---------------------------------------------------------------------------
// Owner mode: split-phase instance barrier.  Every CTA of an instance arrives
// once per step (release), and waits (acquire) until all have arrived for a
// given step; the arrival count of step t is (t + 1 - ts_base) * n_cta.  In
// cluster mode the hardware cluster barrier is used in the same arrive / wait
// order (each arrive is followed by exactly one wait).  Waits are bounded.
// ---------------------------------------------------------------------------
__device__ __forceinline__ void b200_owner_arrive(const b200_inst_d& I, int cluster) {
  __syncthreads();
  if (cluster) {
    asm volatile("barrier.cluster.arrive.release.aligned;\n" ::: "memory");
    return;
  }
  if (threadIdx.x == 0) {
    __threadfence();  // (the fence releases the CTA's writes; the add itself can be relaxed)
    b200_red_relaxed_add64(I.bar64, 1ull);
  }
}

__device__ __forceinline__ bool b200_owner_wait(const b200_inst_d& I, int64_t t, uint64_t limit_ns,
                                                int cluster) {
  if (cluster) {
    asm volatile("barrier.cluster.wait.acquire.aligned;\n" ::: "memory");
    return true;
  }
  __shared__ int ok;
  if (threadIdx.x == 0) {
    ok = 1;
    const unsigned long long target = (unsigned long long)(t + 1 - I.ts_base) * (unsigned long long)I.n_cta;
    if (b200_ld_acquire64(I.bar64) < target) {
      const uint64_t t0 = b200_globaltimer();
      int spins = 0;
      while (b200_ld_acquire64(I.bar64) < target) {
        if (++spins > 32) __nanosleep(32);
        if ((spins & 255) == 0 &&
            (b200_globaltimer() - t0 > limit_ns || *((volatile int32_t*)I.status) != 0)) {
          atomicCAS(I.status, 0, B200_ERR_BARRIER_TIMEOUT);
          ok = 0;
          break;
        }
      }
    }
  }
  __syncthreads();
  return ok != 0;
}

// ---------------------------------------------------------------------------
// Owner mode: relayout of one pathway's CSR over (source, delay slot) into
// segments over (source, owning CTA), stable (within a segment the synapses
// keep their (delay, CSR) order).  One warp per source; `own_lo` [n_own + 1]
// are the first target neurons owned by each CTA.  Every source's synapses
// stay in the source's range of the CSR, so oseg[s * n_own + r] starts at
// segptr[s * W] plus the counts of the owners before r.  `cnt` is n_own ints of
// shared memory per warp.
// ---------------------------------------------------------------------------
struct b200_relayout_args {
  const int64_t* segptr;   // [n_src * W + 1]
  const int32_t* post;     // [n_syn]
  const void* var[B200_MAX_PAYLOAD];
  int32_t var_size[B200_MAX_PAYLOAD];
  int32_t n_var;
  int32_t n_src, W, dmin, n_own;
  const int32_t* own_lo;   // [n_own + 1]
  int64_t* oseg;           // [n_src * n_own + 1]
  int32_t* opost;          // [n_syn]
  uint16_t* odelay;        // [n_syn]
  void* ovar[B200_MAX_PAYLOAD];
  int32_t* status;         // set to B200_ERR_INDEX on an out-of-range target
  unsigned long long* own_in;  // [n_own] incoming synapses per owner (accumulated)
};

__device__ __forceinline__ int b200_owner_of(const int32_t* own_lo, int n_own, int32_t t) {
  int lo = 0, hi = n_own;  // last r with own_lo[r] <= t
  while (hi - lo > 1) {
    const int m = (lo + hi) >> 1;
    if (own_lo[m] <= t) lo = m; else hi = m;
  }
  return lo;
}

__global__ void b200_owner_relayout_kernel(b200_relayout_args A) {
  extern __shared__ int b200_rl_smem[];
  int* s_own = b200_rl_smem;                                     // [n_own + 1]
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nwarp = blockDim.x >> 5;
  int* cnt = b200_rl_smem + A.n_own + 1 + wid * A.n_own;        // [n_own] per warp
  // [n_own] per warp: this warp's synapses per owner (8-byte aligned after the int arrays)
  unsigned long long* tot = (unsigned long long*)(b200_rl_smem + ((A.n_own + 1 + nwarp * A.n_own + 1) & ~1)) +
                            (size_t)wid * A.n_own;
  for (int k = threadIdx.x; k <= A.n_own; k += blockDim.x) s_own[k] = A.own_lo[k];
  for (int k = lane; k < A.n_own; k += 32) tot[k] = 0;
  __syncthreads();
  const int32_t t_lo = s_own[0], t_hi = s_own[A.n_own];
  for (int64_t s = (int64_t)blockIdx.x * nwarp + wid; s < A.n_src; s += (int64_t)gridDim.x * nwarp) {
    const int64_t* sp = A.segptr + s * A.W;
    const int64_t base = sp[0], end = sp[A.W];
    for (int r = lane; r < A.n_own; r += 32) cnt[r] = 0;
    __syncwarp();
    // pass 1: synapses per owner
    for (int64_t j0 = base; j0 < end; j0 += 32) {
      const int64_t j = j0 + lane;
      if (j < end) {
        const int32_t t = A.post[j];
        if (t < t_lo || t >= t_hi) atomicCAS(A.status, 0, B200_ERR_INDEX);
        else atomicAdd(&cnt[b200_owner_of(s_own, A.n_own, t)], 1);
      }
    }
    __syncwarp();
    // exclusive prefix over owners (serial per warp lane 0: n_own is small)
    if (lane == 0) {
      int64_t acc = 0;
      for (int r = 0; r < A.n_own; ++r) {
        const int c = cnt[r];
        A.oseg[s * A.n_own + r] = base + acc;
        cnt[r] = (int)acc;
        acc += c;
        tot[r] += (unsigned long long)c;
      }
    }
    __syncwarp();
    // pass 2: stable scatter, delay slot by delay slot
    for (int k = 0; k < A.W; ++k) {
      const int64_t a = sp[k], b = sp[k + 1];
      for (int64_t j0 = a; j0 < b; j0 += 32) {
        const int64_t j = j0 + lane;
        const bool act = j < b;
        int32_t t = 0;
        int r = -1;
        if (act) {
          t = A.post[j];
          if (t >= t_lo && t < t_hi) r = b200_owner_of(s_own, A.n_own, t);
        }
        const unsigned peers = __match_any_sync(0xffffffffu, r);
        const int rank = __popc(peers & b200_lanemask_lt());
        const int c0 = r >= 0 ? cnt[r] : 0;
        __syncwarp();
        if (r >= 0) {
          const int64_t pos = base + c0 + rank;
          A.opost[pos] = t;
          A.odelay[pos] = (uint16_t)(A.dmin + k);
          for (int v = 0; v < A.n_var; ++v) {
            if (A.var_size[v] == 8)
              ((int64_t*)A.ovar[v])[pos] = ((const int64_t*)A.var[v])[j];
            else
              ((int32_t*)A.ovar[v])[pos] = ((const int32_t*)A.var[v])[j];
          }
          if (rank == 0) cnt[r] = c0 + __popc(peers);
        }
        __syncwarp();
      }
    }
    __syncwarp();
  }
  __syncwarp();
  for (int k = lane; k < A.n_own; k += 32)
    if (tot[k]) atomicAdd(&A.own_in[k], tot[k]);
  if (blockIdx.x == 0 && threadIdx.x == 0) A.oseg[(int64_t)A.n_src * A.n_own] = A.segptr[(int64_t)A.n_src * A.W];
}
