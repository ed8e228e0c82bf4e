/*
 * b200_peaks.h -- measured arithmetic peaks of the device (libb200_peaks,
 * brian2_gb300/csrc/b200_peaks.cu).
 *
 * No counterpart in the reference (it has no GPU code): the denominators of
 * the ALU roofline of compute-bound step loops (Hodgkin-Huxley networks),
 * measured on the device rather than taken from a data sheet.
 */
#ifndef B200_PEAKS_H
#define B200_PEAKS_H
#include <stdint.h>
#ifdef __cplusplus
extern "C" {
#endif
const char* b200p_last_error(void);
/* Throughput of fused multiply-adds on every SM (8 independent chains per
 * thread, `iterations` x 64 FMAs each), float64 when fp64 != 0, else float32:
 * *gflops in GFLOP/s (2 flops per FMA, best of three timed launches after a
 * warm-up), *ms the best launch's duration (may be NULL).  0 on success. */
int b200p_fma_peak(int32_t fp64, int64_t iterations, double* gflops, double* ms);
#ifdef __cplusplus
}
#endif
#endif
