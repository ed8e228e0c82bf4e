/*
 * b200.h -- C ABI of the GB300 clock-driven step engine for Brian2.
 *
 * Every model library (one per network spec, built by brian2_gb300.native from
 * the code generator's output) exports exactly these symbols.  Plain C types
 * only; the handle owns all device memory; every entry point returns a status
 * (0 = ok, see B200_STATUS_*) and b200_last_error() gives the message.  No entry
 * point calls exit(): the reference's generated code exits on bad sizes or
 * indices (brian2/devices/cpp_standalone/templates/synapses_create_generator.cpp:105,113,196,218),
 * here those are B200_STATUS_INDEX / B200_STATUS_ARG.
 *
 * The reference has no C ABI for this path: its boundary is "generate a C++
 * project and run ./main" (brian2/devices/cpp_standalone/device.py:1207-1351).
 * Each function below names the piece of that project it replaces.
 */
#ifndef B200_H
#define B200_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct b200_net b200_net;

#define B200_STATUS_OK 0
#define B200_STATUS_CUDA 1     /* a CUDA runtime call failed */
#define B200_STATUS_ARG 2      /* invalid argument (sizes, ranges, ids) */
#define B200_STATUS_CAPACITY 3 /* a buffer limit was exceeded */
#define B200_STATUS_TIMEOUT 4  /* a bounded device-side wait gave up */
#define B200_STATUS_INDEX 5    /* an index (synapse, neuron) out of range */
#define B200_STATUS_RANDOM 6   /* a draw needed more random numbers than the stream's layout gives
                                  (a rejected binomial draw of a Poisson input, probability < 1e-15) */

/* Kinds of variables addressed by b200_upload / b200_download. */
#define B200_VAR_GROUP 0   /* neuron-group state variable */
#define B200_VAR_SYNAPSE 1 /* synaptic variable, given in synapse creation order */

/* Creates n_inst independent instances of the model (one network, or a batched
 * sweep).  group_sizes[k*n_groups+g] = neurons of group g in instance k.
 * Replaces _init_arrays (brian2/devices/cpp_standalone/templates/objects.cpp:185-248). */
int b200_create(b200_net** out, int32_t n_inst, const int32_t* group_sizes, double dt);
/* Frees every device buffer of the handle. Replaces _dealloc_arrays (objects.cpp:372-400). */
int b200_destroy(b200_net* net);
/* Copies the message of the last failing call into buf. */
int b200_last_error(b200_net* net, char* buf, int64_t len);

/* Launch shape: threads per CTA, CTAs per instance (>1: instance barrier), queue
 * mode (resident CTAs pull single-CTA instances), steps per kernel launch, and
 * whether launches are replayed from a captured CUDA graph.  Replaces the OpenMP
 * thread preference (brian2/devices/cpp_standalone/device.py:60-67). */
int b200_configure(b200_net* net, int32_t threads, const int32_t* ctas_per_inst, int32_t queue_mode,
                   int64_t chunk_steps, int32_t use_graph);
/* Keep the state of single-CTA instances, and each CTA's own neurons' private
 * variables (those no pathway touches) in multi-CTA instances, in shared memory
 * for the duration of a launch (default on; off is for comparison and tuning). */
int b200_set_smem_cache(b200_net* net, int32_t enable);
/* Run instances of 2..16 CTAs as thread-block clusters with the hardware cluster
 * barrier (default on), and report the launch plan that b200_run will use. */
int b200_set_clusters(b200_net* net, int32_t enable);
int b200_launch_plan(b200_net* net, int32_t* grid, int32_t* cluster, int32_t* state_bytes);
/* Owner-mode delivery (0 off, 1 on where it applies, 2 auto = default: on for
 * networks without synaptic delays, where it is measured faster): each CTA of a multi-CTA
 * instance delivers only into the target neurons it owns, keeping their state
 * in shared memory, with per-CTA event FIFOs ordered by due step.  A second
 * implementation of CSpikeQueue + on_pre (brian2/synapses/spikequeue.h:14-206,
 * templates/synapses.cpp:20-49); b200_owner_active reports whether the current
 * launch plan uses it.  The FIFOs default to the worst case (dmax + 2 steps of
 * a CTA's incoming synapses) where that fits in an eighth of the device memory;
 * b200_set_event_capacity sizes them in units of a CTA's incoming synapses
 * instead.  An overflow fails the run with B200_STATUS_CAPACITY and a message. */
int b200_set_owner(b200_net* net, int32_t enable);
int b200_owner_active(b200_net* net, int32_t* active);
int b200_set_event_capacity(b200_net* net, double factor);
/* Push-mode delivery (0 off, 1 on where it applies, 2 auto = default: on for
 * float32 models with synaptic delays on instances of 2+ CTAs).  A third
 * implementation of CSpikeQueue + on_pre (brian2/synapses/spikequeue.h:14-206,
 * templates/synapses.cpp:20-49) for models whose on_pre only adds into target
 * variables and whose delays are all >= 1 step: each CTA delivers the spikes of
 * the neurons it owns one step ahead into accumulator buffers that the target's
 * owner adds to its state after the next barrier -- one barrier per step, no
 * global spike list.  The deliveries of a step are summed before they reach
 * their variable, so float64 results may differ from the reference in the last
 * bits (float64 models use it only when asked: 1).  b200_push_active reports
 * whether the current launch plan uses it; it takes precedence over owner mode. */
int b200_set_push(b200_net* net, int32_t enable);
int b200_push_active(b200_net* net, int32_t* active);
/* Spike generator groups (input/spikegeneratorgroup.py:37-372, stepped by
 * templates/spikegenerator.cpp:5-31): the entries' time bins (sorted, the
 * group's `_timebins`), their neuron indices (`neuron_index`), the period in
 * bins (`_period_bins`, 0 = none) and the cursor (`_lastindex`).  Each step
 * emits the entries from the cursor whose bin is <= the step (modulo the
 * period), as the group's spikes.  b200_get_generator reads the cursor back. */
int b200_set_generator(b200_net* net, int32_t inst, int32_t group, const int32_t* bins, const int32_t* index,
                       int64_t count, int32_t period_bins, int32_t last);
int b200_get_generator(b200_net* net, int32_t inst, int32_t group, int32_t* last);
/* The random generator of the step loop, for models that draw in it: rand() in
 * threshold code (PoissonGroup, brian2/input/poissongroup.py), randn() in state
 * updates (stochastic equations, brian2/stateupdaters/explicit.py), the binomial
 * counts of Poisson inputs (brian2/input/poissoninput.py, binomial.py:93-141):
 * the reference's MT19937 state as the C++ library stores it (624 words, then
 * the position), taken where the standalone program starts the run
 * (brian::_random_generators[0], templates/objects.cpp:426-478).  The device
 * continues that stream in the reference's order of draws (code objects in
 * schedule order, neurons in index order; rand() = (a*2^26 + b)/2^53 of two
 * outputs; randn() by the polar method).
 * b200_get_rng returns the generator state and the steps of words generated
 * ahead of the current step. */
int b200_set_rng(b200_net* net, int32_t inst, const uint32_t* words, int32_t position);
int b200_get_rng(b200_net* net, int32_t inst, uint32_t* words, int32_t* position, int64_t* unused_steps);
/* randn()'s kept value (objects.cpp:455-477: the polar method returns one value
 * of each accepted pair and keeps the other for the next call): set after
 * b200_set_rng when the program had one kept where the run starts. */
int b200_set_rng_gauss(b200_net* net, int32_t inst, int32_t has, double value);
int b200_get_rng_gauss(b200_net* net, int32_t inst, int32_t* has, double* value);
/* Per-instance values of the model's namespace constants (the %CONSTANTS% of the
 * generated code objects, device.py:936-940); scalar blocks are re-evaluated. */
int b200_set_consts(b200_net* net, int32_t inst, const double* values, int32_t count);

/* Host <-> device copies of state and synaptic variables.
 * Replace _load_arrays / _write_arrays (objects.cpp:249-370). */
int b200_upload(b200_net* net, int32_t inst, int32_t kind, int32_t obj, int32_t var, const void* src,
                int64_t count);
int b200_download(b200_net* net, int32_t inst, int32_t kind, int32_t obj, int32_t var, void* dst,
                  int64_t count);

/* Synapses of one pathway in creation order.  pre/post are relative to the source
 * range [src_lo,src_hi) and target range [tgt_lo,tgt_hi); delay_steps[k] is the
 * quantised delay (int)(delay/dt+0.5), or NULL for the single scalar_delay.
 * Replaces CSpikeQueue::prepare (brian2/synapses/spikequeue.h:45-105) and the
 * before_run block of templates/synapses_push_spikes.cpp:5-17. */
int b200_set_synapses(b200_net* net, int32_t inst, int32_t pathway, int32_t src_lo, int32_t src_hi,
                      int32_t tgt_lo, int32_t tgt_hi, const int32_t* pre, const int32_t* post,
                      const int32_t* delay_steps, int32_t scalar_delay, int64_t n_syn);
/* Same, from a CSR over (source, delay slot) that is already in device memory
 * (device-side construction of very large networks). */
int b200_set_synapses_csr(b200_net* net, int32_t inst, int32_t pathway, int32_t src_lo, int32_t src_hi,
                          int32_t tgt_lo, int32_t tgt_hi, int32_t dmin, int32_t dmax,
                          const int64_t* d_segptr, const int32_t* d_post, const int32_t* d_pre,
                          int64_t n_syn);
/* Device address of a synaptic variable (CSR order) for device-side fills. */
int b200_synapse_var_ptr(b200_net* net, int32_t inst, int32_t pathway, int32_t var, void** out);

/* Monitor ranges (subgroup sources) and StateMonitor selection.  Replace the
 * _source_start/_source_stop handling of templates/spikemonitor.cpp:17-33,
 * templates/ratemonitor.cpp:8-31 and the record indices of templates/statemonitor.cpp. */
int b200_set_monitor_range(b200_net* net, int32_t inst, int32_t kind, int32_t mon, int32_t lo, int32_t hi);
int b200_set_statemon(b200_net* net, int32_t inst, int32_t mon, const int32_t* idx, int32_t n_rec,
                      const int32_t* vars, int32_t n_vars);

/* Runs every instance n_steps clock steps from its current step: state update,
 * threshold, spike monitor, propagation (advance/push/on_pre), reset, rate and
 * state monitors, clock tick -- all on the device.  Replaces Network::run
 * (templates/network.cpp:38-122) with the code objects of stateupdate.cpp,
 * threshold.cpp, spikemonitor.cpp, synapses_push_spikes.cpp, synapses.cpp,
 * reset.cpp, ratemonitor.cpp and statemonitor.cpp. */
int b200_run(b200_net* net, int64_t n_steps);
/* Current clock step of an instance (Clock::timestep, brianlib/clocks.h:34-38). */
int b200_get_step(b200_net* net, int32_t inst, int64_t* ts);
/* Sets an instance's clock step.  After a run that failed part-way (timeout,
 * index error, dropped events) the instance's CTAs stopped at different steps
 * and b200_run refuses it (B200_STATUS_ARG) until the caller has uploaded a
 * consistent state and declared its step here. */
int b200_set_step(b200_net* net, int32_t inst, int64_t ts);
/* Device time of the last b200_run in ms (CUDA events); the reference's
 * _last_run_time (device.py:1326-1332). */
int b200_last_run_ms(b200_net* net, double* ms);
/* Device time of the step-kernel launches of the last b200_run only, in ms. */
int b200_last_kernel_ms(b200_net* net, double* ms);

/* Monitor contents, copied back on request (device-resident until then).
 * Replace the dynamic arrays written by spikemonitor.cpp:37-47, ratemonitor.cpp:33-35,
 * statemonitor.cpp. */
int b200_spikemon_size(b200_net* net, int32_t inst, int32_t mon, int64_t* count);
int b200_spikemon_get(b200_net* net, int32_t inst, int32_t mon, int32_t* i, int32_t* ts,
                      int32_t* per_neuron, int64_t count);
/* The values of a spike monitor's recorded variables (SpikeMonitor(G, variables=...),
 * monitors/spikemonitor.py:62-67; appended with i and t by spikemonitor.cpp:37-47):
 * vals[count][n_vars] as double, in the order of the spikes, each the
 * variable's value when the step's thresholder ran (after the state update,
 * before that step's deliveries and reset).  n_vars is the model's count for
 * that monitor; count as from b200_spikemon_size. */
int b200_spikemon_values(b200_net* net, int32_t inst, int32_t mon, double* vals, int64_t count);
int b200_ratemon_size(b200_net* net, int32_t inst, int32_t mon, int64_t* steps);
int b200_ratemon_get(b200_net* net, int32_t inst, int32_t mon, int32_t* counts, int64_t steps);
int b200_statemon_size(b200_net* net, int32_t inst, int32_t mon, int64_t* steps);
int b200_statemon_get(b200_net* net, int32_t inst, int32_t mon, double* data, int64_t steps);
int b200_reset_monitors(b200_net* net, int32_t inst);

/* Bounded device-side waits: limit in ns for the instance barrier, and a test
 * hook (fault_rank >= 0) that makes that CTA leave before its first barrier of
 * the next launch, so the others time out and b200_run returns
 * B200_STATUS_TIMEOUT with the handle still usable (every instance's status and
 * barrier words are cleared; a failed instance runs again after
 * b200_set_step).  The reference's analogue
 * is the wall-clock limit of Network::run (templates/network.cpp:59-82). */
int b200_set_wait_limit(b200_net* net, int64_t limit_ns, int32_t fault_rank);

/* Per-phase device profile of the step kernel (SM cycles summed over CTAs and
 * steps; phases: update/threshold/reset, barrier, spike lists and monitors, one
 * per pathway, barrier).  Replaces run(profile=True) timing
 * (templates/common_group.cpp:72-90, objects.cpp:351-358). */
int b200_set_profiling(b200_net* net, int32_t enable);
int b200_profile_phases(b200_net* net, int32_t* count);
int b200_get_profile(b200_net* net, int32_t inst, uint64_t* cycles, int32_t n_phases);

/* Introspection. */
int b200_model_name(char* buf, int64_t len);
int b200_device_bytes(b200_net* net, int64_t* bytes);
int b200_launch_count(b200_net* net, int64_t* count);

#ifdef __cplusplus
}
#endif
#endif /* B200_H */
