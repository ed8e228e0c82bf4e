// Host-side network construction with Brian2's cpp_standalone random stream.
//
// Brian's standalone device draws every random number of initialisation and
// synapse creation from one mt19937 per thread, seeded `seed + thread`
// (brian2/devices/cpp_standalone/device.py:873-884), and combines two 32-bit
// outputs into a 53-bit double (templates/objects.cpp:448-453).  `randn()` is
// the polar Box-Muller method that caches its second value
// (templates/objects.cpp:455-469).  Reproducing the same stream, in the same
// draw order, is what makes constructed networks identical to the reference's
// (checked against digests of the reference's own synapse arrays).
//
// The generator is MT19937 as published by Matsumoto & Nishimura (1998),
// written here from the published recurrence; seeding is the published
// init_genrand.  Compile with -ffp-contract=off so that log/floor arithmetic is
// evaluated exactly as in the reference build.
#include <cmath>
#include <cstdint>
#include <cstring>
#include <set>
#include <vector>

extern "C" {

struct b200_rng {
  uint32_t mt[624];
  int32_t idx;
  int32_t has_gauss;
  double gauss;
};

void b200_rng_seed(b200_rng* r, uint32_t seed) {
  r->mt[0] = seed;
  for (int i = 1; i < 624; ++i)
    r->mt[i] = 1812433253u * (r->mt[i - 1] ^ (r->mt[i - 1] >> 30)) + (uint32_t)i;
  r->idx = 624;
  r->has_gauss = 0;
  r->gauss = 0.0;
}

static inline uint32_t b200_mt_next(b200_rng* r) {
  if (r->idx >= 624) {
    for (int i = 0; i < 624; ++i) {
      const uint32_t y = (r->mt[i] & 0x80000000u) | (r->mt[(i + 1) % 624] & 0x7fffffffu);
      uint32_t v = r->mt[(i + 397) % 624] ^ (y >> 1);
      if (y & 1u) v ^= 0x9908b0dfu;
      r->mt[i] = v;
    }
    r->idx = 0;
  }
  uint32_t y = r->mt[r->idx++];
  y ^= (y >> 11);
  y ^= (y << 7) & 0x9d2c5680u;
  y ^= (y << 15) & 0xefc60000u;
  y ^= (y >> 18);
  return y;
}

uint32_t b200_rng_u32(b200_rng* r) { return b200_mt_next(r); }

// 53-bit uniform in [0,1): ((a>>5)*2^26 + (b>>6)) / 2^53
double b200_rng_rand(b200_rng* r) {
  const long a = (long)(b200_mt_next(r) >> 5);
  const long b = (long)(b200_mt_next(r) >> 6);
  return (a * 67108864.0 + b) / 9007199254740992.0;
}

double b200_rng_randn(b200_rng* r) {
  if (r->has_gauss) {
    r->has_gauss = 0;
    return r->gauss;
  }
  double f, x1, x2, r2;
  do {
    x1 = 2.0 * b200_rng_rand(r) - 1.0;
    x2 = 2.0 * b200_rng_rand(r) - 1.0;
    r2 = x1 * x1 + x2 * x2;
  } while (r2 >= 1.0 || r2 == 0.0);
  f = sqrt(-2.0 * log(r2) / r2);
  r->gauss = f * x1;
  r->has_gauss = 1;
  return f * x2;
}

void b200_rng_fill_rand(b200_rng* r, double* out, int64_t n) {
  for (int64_t k = 0; k < n; ++k) out[k] = b200_rng_rand(r);
}
void b200_rng_fill_randn(b200_rng* r, double* out, int64_t n) {
  for (int64_t k = 0; k < n; ++k) out[k] = b200_rng_randn(r);
}

// `x = a + b*rand()` for n values in order (the form Brian generates for
// `x = 'a + rand()*b'` after loop-invariant hoisting of b).
void b200_rng_affine_rand(b200_rng* r, double a, double b, double* out, int64_t n) {
  for (int64_t k = 0; k < n; ++k) out[k] = a + (b * b200_rng_rand(r));
}

// `x = a + (scale * (c0 + (c1 * randn())))` for n values in order.
void b200_rng_affine_randn(b200_rng* r, double a, double scale, double c0, double c1, double* out,
                           int64_t n) {
  for (int64_t k = 0; k < n; ++k) out[k] = a + (scale * (c0 + (c1 * b200_rng_randn(r))));
}

// Bernoulli connection `connect(condition, p=p)`
// (templates/synapses_create_generator.cpp:155-171 jump algorithm for p<0.25,
// per-candidate test otherwise).  Outer loop over presynaptic i in
// [0, n_pre); inner candidates j in [0, n_post).  The condition is
// `i_lo <= i < i_hi` (and `i != j` when no_self).  When `cond_uses_j` is 0 the
// condition is tested before the inner loop (no random numbers are drawn for
// rejected i), as Brian does for conditions that do not depend on j; otherwise
// every i draws and each candidate is tested after its draw.
// Returns the number of synapses written, or -1 if `cap` is too small.
int64_t b200_connect_bernoulli(b200_rng* r, int32_t n_pre, int32_t n_post, double p, int32_t i_lo,
                               int32_t i_hi, int32_t no_self, int32_t cond_uses_j, int32_t* pre_out,
                               int32_t* post_out, int64_t cap) {
  int64_t n = 0;
  for (int32_t i = 0; i < n_pre; ++i) {
    const bool i_ok = (i >= i_lo && i < i_hi);
    if (!cond_uses_j && !i_ok) continue;
    if (p == 0) continue;
    const bool jump_algo = p < 0.25;
    const double pconst = 1.0 / log(1 - p);
    for (long k = 0; k < n_post; k += 1) {
      if (jump_algo) {
        const double u = b200_rng_rand(r);
        if (u == 0.0) break;
        const int jump = (int)(floor(log(u) * pconst) * 1);
        k += jump;
        if (k >= n_post) continue;
      } else {
        if (b200_rng_rand(r) >= p) continue;
      }
      if (!i_ok) continue;
      if (no_self && (long)i == k) continue;
      if (n >= cap) return -1;
      pre_out[n] = i;
      post_out[n] = (int32_t)k;
      ++n;
    }
  }
  return n;
}

// Fixed in-degree `connect(i='k for k in sample(N_pre, size=K)')`: outer loop
// over postsynaptic j, inner sample of K distinct presynaptic indices
// (templates/synapses_create_generator.cpp:85-153): selection sampling
// (Knuth, TAOCP vol. 2, 3.4.2, algorithm S) when K/n > 0.06, otherwise
// rejection into an ordered set, emitted in ascending order.
int64_t b200_connect_fixed_indegree(b200_rng* r, int32_t n_pre, int32_t n_post, int32_t K,
                                    int32_t* pre_out, int32_t* post_out, int64_t cap) {
  int64_t n = 0;
  if (K > n_pre || K < 0) return -2;
  const int n_total = n_pre;
  const bool selection = 1.0 * K / n_total > 0.06;
  std::set<int> chosen;
  for (int32_t j = 0; j < n_post; ++j) {
    if (K == 0) continue;
    int n_selected = 0, n_dealt_with = 0;
    long k;
    std::set<int>::iterator it;
    if (selection) {
      k = -1;
    } else {
      chosen.clear();
      while (n_selected < K) {
        int v = (int)(b200_rng_rand(r) * n_total);
        while (!chosen.insert(v).second) v = (int)(b200_rng_rand(r) * n_total);
        n_selected++;
      }
      n_selected = 0;
      it = chosen.begin();
    }
    while (n_selected < K) {
      if (selection) {
        k += 1;
        n_dealt_with++;
        const double U = b200_rng_rand(r);
        if ((n_total - n_dealt_with) * U >= (long)K - n_selected) continue;
      } else {
        k = *it;
        ++it;
      }
      n_selected++;
      if (n >= cap) return -1;
      pre_out[n] = (int32_t)k;
      post_out[n] = j;
      ++n;
    }
  }
  return n;
}

// Quantised delays as CSpikeQueue::prepare computes them:
// (int)(delay/dt + 0.5)  (brian2/synapses/spikequeue.h:85-95)
void b200_quantise_delays(const double* delay, int64_t n, double dt, int32_t* out) {
  for (int64_t k = 0; k < n; ++k) out[k] = (int)(delay[k] / dt + 0.5);
}
void b200_quantise_delays_f32(const float* delay, int64_t n, double dt, int32_t* out) {
  for (int64_t k = 0; k < n; ++k) out[k] = (int)(delay[k] / dt + 0.5);
}

}  // extern "C"
