/*
 * THE ORACLE -- test infrastructure only.
 *
 * CPU restatement of the device construction of fixed in-degree networks
 * (brian2_gb300/csrc/b200_scale.cu), written independently in plain C so the
 * GPU result can be checked bit for bit: Philox4x32-10 (Salmon et al., SC'11),
 * K distinct sources per target by sort-and-redraw, delay slots
 * (int)((dmin + dspan*U53)/dt + 0.5) as CSpikeQueue::prepare quantises
 * (brian2/synapses/spikequeue.h:85-95), and a CSR over (source, slot) whose
 * segments hold targets in ascending order.
 */
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

static void philox(uint32_t c[4], uint32_t k0, uint32_t k1) {
  for (int r = 0; r < 10; ++r) {
    uint64_t p0 = (uint64_t)0xD2511F53u * c[0];
    uint64_t p1 = (uint64_t)0xCD9E8D57u * c[2];
    uint32_t n0 = (uint32_t)(p1 >> 32) ^ c[1] ^ k0;
    uint32_t n1 = (uint32_t)p1;
    uint32_t n2 = (uint32_t)(p0 >> 32) ^ c[3] ^ k1;
    uint32_t n3 = (uint32_t)p0;
    c[0] = n0; c[1] = n1; c[2] = n2; c[3] = n3;
    k0 += 0x9E3779B9u;
    k1 += 0xBB67AE85u;
  }
}

static uint32_t draw(uint32_t k, uint32_t j, uint32_t p, uint32_t r, uint64_t seed, uint32_t M) {
  uint32_t c[4] = {k, j, p, r};
  philox(c, (uint32_t)seed, (uint32_t)(seed >> 32));
  return (uint32_t)(((uint64_t)c[0] * (uint64_t)M) >> 32);
}

static double u53(uint32_t k, uint32_t j, uint32_t p, uint64_t seed) {
  uint32_t c[4] = {k, j, p, 255u};
  philox(c, (uint32_t)seed, (uint32_t)(seed >> 32));
  long a = (long)(c[0] >> 5), b = (long)(c[1] >> 6);
  return (a * 67108864.0 + b) / 9007199254740992.0;
}

static int cmp_u32(const void* a, const void* b) {
  uint32_t x = *(const uint32_t*)a, y = *(const uint32_t*)b;
  return x < y ? -1 : x > y;
}

/* pre/slot in target-major order (n_post*K); returns 0 on success */
int scale_ref_sample(uint64_t seed, uint32_t p, uint32_t M, int K, int n_post, double dmin, double dspan,
                     double dt, int32_t* pre, int32_t* slot) {
  uint32_t* v = (uint32_t*)malloc(sizeof(uint32_t) * (K > 0 ? K : 1));
  unsigned char* dup = (unsigned char*)malloc(K > 0 ? K : 1);
  for (int j = 0; j < n_post; ++j) {
    if ((int64_t)K * 16 > (int64_t)M) {
      /* dense: Knuth's selection sampling, in Brian's form */
      int sel = 0;
      for (uint32_t c = 0; c < M && sel < K; ++c) {
        double U = u53(c, (uint32_t)j, p + 1024u, seed);
        if ((double)(M - (c + 1)) * U < (double)(K - sel)) v[sel++] = c;
      }
      goto emit;
    }
    for (int k = 0; k < K; ++k) v[k] = draw((uint32_t)k, (uint32_t)j, p, 0u, seed, M);
    int round;
    for (round = 1; round <= 64; ++round) {
      qsort(v, K, sizeof(uint32_t), cmp_u32);
      int any = 0;
      for (int k = 0; k < K; ++k) dup[k] = (k > 0 && v[k] == v[k - 1]);
      for (int k = 0; k < K; ++k)
        if (dup[k]) { v[k] = draw((uint32_t)k, (uint32_t)j, p, (uint32_t)round, seed, M); any = 1; }
      if (!any) break;
      if (round == 64) { free(v); free(dup); return 1; }
    }
  emit:
    for (int k = 0; k < K; ++k) {
      pre[(int64_t)j * K + k] = (int32_t)v[k];
      double d = dmin + dspan * u53((uint32_t)k, (uint32_t)j, p, seed);
      slot[(int64_t)j * K + k] = (int)(d / dt + 0.5);
    }
  }
  free(v);
  free(dup);
  return 0;
}

/* stable counting sort into a CSR over (source, slot - s0); targets ascend
   within a segment because targets are visited in ascending order */
void scale_ref_csr(const int32_t* pre, const int32_t* slot, int64_t n, int K, int n_src, int s0, int W,
                   int src_off, int64_t* seg, int32_t* post_csr, int32_t* pre_csr) {
  int64_t nb = (int64_t)n_src * W;
  memset(seg, 0, sizeof(int64_t) * (nb + 1));
  for (int64_t e = 0; e < n; ++e) seg[(int64_t)pre[e] * W + (slot[e] - s0) + 1]++;
  for (int64_t b = 0; b < nb; ++b) seg[b + 1] += seg[b];
  int64_t* fill = (int64_t*)malloc(sizeof(int64_t) * (nb > 0 ? nb : 1));
  memcpy(fill, seg, sizeof(int64_t) * nb);
  for (int64_t e = 0; e < n; ++e) {
    int64_t b = (int64_t)pre[e] * W + (slot[e] - s0);
    int64_t pos = fill[b]++;
    post_csr[pos] = (int32_t)(e / K);
    pre_csr[pos] = (int32_t)(b / W) + src_off;
  }
  free(fill);
}
