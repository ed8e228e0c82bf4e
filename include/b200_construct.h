/*
 * b200_construct.h -- host construction with Brian2's standalone random stream
 * (libb200_construct, built from brian2_gb300/csrc/b200_construct.cpp).
 *
 * Reproduces, draw for draw, the random numbers a single-threaded Brian2
 * cpp_standalone program takes after seed(s): mt19937 seeded s
 * (brian2/devices/cpp_standalone/device.py:873-884), rand() from two 32-bit
 * draws (templates/objects.cpp:448-453), polar randn() with its cached value
 * (templates/objects.cpp:455-469), and the synapse generator loops of
 * templates/synapses_create_generator.cpp.
 */
#ifndef B200_CONSTRUCT_H
#define B200_CONSTRUCT_H
#include <stdint.h>
#ifdef __cplusplus
extern "C" {
#endif

typedef struct b200_rng {
  uint32_t mt[624];
  int32_t idx;
  int32_t has_gauss;
  double gauss;
} b200_rng;

/* RandomGenerator::seed(unsigned long) (objects.cpp:436-439) */
void b200_rng_seed(b200_rng* r, uint32_t seed);
uint32_t b200_rng_u32(b200_rng* r);
/* RandomGenerator::rand() (objects.cpp:448-453) */
double b200_rng_rand(b200_rng* r);
/* RandomGenerator::randn() (objects.cpp:455-469) */
double b200_rng_randn(b200_rng* r);
void b200_rng_fill_rand(b200_rng* r, double* out, int64_t n);
void b200_rng_fill_randn(b200_rng* r, double* out, int64_t n);
/* n values of a + (b * rand()) -- group_variable_set_conditional for 'a + rand()*b' */
void b200_rng_affine_rand(b200_rng* r, double a, double b, double* out, int64_t n);
/* n values of a + (scale * (c0 + (c1 * randn()))) */
void b200_rng_affine_randn(b200_rng* r, double a, double scale, double c0, double c1, double* out, int64_t n);
/* connect(condition, p=p) -- synapses_create_generator.cpp:155-171 (jump algorithm) */
int64_t b200_connect_bernoulli(b200_rng* r, int32_t n_pre, int32_t n_post, double p, int32_t i_lo,
                               int32_t i_hi, int32_t no_self, int32_t cond_uses_j, int32_t* pre_out,
                               int32_t* post_out, int64_t cap);
/* connect(i='k for k in sample(N_pre, size=K)') -- synapses_create_generator.cpp:85-153 */
int64_t b200_connect_fixed_indegree(b200_rng* r, int32_t n_pre, int32_t n_post, int32_t K,
                                    int32_t* pre_out, int32_t* post_out, int64_t cap);
/* (int)(delay/dt + 0.5) -- CSpikeQueue::prepare (brian2/synapses/spikequeue.h:85-95) */
void b200_quantise_delays(const double* delay, int64_t n, double dt, int32_t* out);
void b200_quantise_delays_f32(const float* delay, int64_t n, double dt, int32_t* out);

#ifdef __cplusplus
}
#endif
#endif
