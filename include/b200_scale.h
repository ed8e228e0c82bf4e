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
uint32_t b200s_host_draw(uint32_t k, uint32_t j, uint32_t p, uint32_t r, uint64_t seed, uint32_t M);
#ifdef __cplusplus
}
#endif
#endif
