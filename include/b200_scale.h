/*
 * b200_scale.h -- device-side construction of large fixed in-degree networks
 * (libb200_scale, brian2_gb300/csrc/b200_scale.cu).
 *
 * Replaces, for networks too large for the host loop, the reference's
 * `connect(i='k for k in sample(N_pre, size=K)')` path
 * (brian2/devices/cpp_standalone/templates/synapses_create_generator.cpp:85-153)
 * and its per-synapse delay draw, with a counter-based generator on the GPU;
 * the result is a CSR over (source, delay slot) ready for b200_set_synapses_csr.
 */
#ifndef B200_SCALE_H
#define B200_SCALE_H
#include <stdint.h>
#ifdef __cplusplus
extern "C" {
#endif
/* Status codes of the b200s_* entry points (message: b200s_last_error()). */
#define B200S_STATUS_OK 0
#define B200S_STATUS_CUDA 1           /* a CUDA runtime call failed */
#define B200S_STATUS_ARG 2            /* invalid sizes, delays or buffers */
#define B200S_STATUS_NOT_CONVERGED 3  /* the source sampling did not converge */
#define B200S_STATUS_INDEX 5          /* construction produced an out-of-range index */
#define B200S_STATUS_SCRATCH_LIMIT 7  /* beyond the allocation-free entry point's scratch array */
const char* b200s_last_error(void);
int b200s_fixed_indegree_csr(uint64_t seed, int32_t path_id, int32_t n_src, int32_t src_off, int32_t n_post,
                             int32_t K, double dmin, double dspan, double dt, int32_t* slot_min,
                             int32_t* slot_max, int64_t** d_segptr, int32_t** d_post, int32_t** d_pre,
                             int64_t* n_syn);
int b200s_free(void* p);
int b200s_fill_f32(float* p, float v, int64_t n);
int b200s_fill_f64(double* p, double v, int64_t n);
int b200s_to_host(void* dst, const void* src, int64_t bytes);
int b200s_outdegree(const int64_t* d_segptr, int32_t n_src, int32_t W, int32_t* host_out);

/* No counterpart in the reference.  Allocation-free variant of
 * b200s_fixed_indegree_csr for callers that may not call cudaMalloc/cudaFree
 * while they run (device memory owned by another framework's pool, or a fixed
 * device-memory budget): outputs are caller-allocated device buffers, the
 * temporaries live in one 16 MiB file-scope device array.  That array belongs
 * to the whole library: loading libb200_scale onto a device reserves its
 * 16 MiB there for the life of the process, whichever entry point is used.
 * Networks needing more scratch are rejected with B200S_STATUS_SCRATCH_LIMIT
 * (a caller may fall back to the allocating entry point on that status
 * alone).  The first call on a device sets up the array's address (make it
 * before any stream capture).  Calls share the array: calls that overlap on
 * the GPU race and must be serialised.  b200s_noalloc_scratch_bytes() gives
 * the scratch a network needs. */
int64_t b200s_noalloc_scratch_bytes(int32_t n_src, int32_t n_post, int32_t K, double dmin, double dspan,
                                    double dt);
int b200s_fixed_indegree_csr_noalloc(uint64_t seed, int32_t path_id, int32_t n_src, int32_t src_off,
                                     int32_t n_post, int32_t K, double dmin, double dspan, double dt,
                                     int32_t* slot_min, int32_t* slot_max, int64_t* d_segptr, int64_t cap_seg,
                                     int32_t* d_post, int32_t* d_pre, int64_t cap_syn);
uint32_t b200s_host_draw(uint32_t k, uint32_t j, uint32_t p, uint32_t r, uint64_t seed, uint32_t M);
#ifdef __cplusplus
}
#endif
#endif
