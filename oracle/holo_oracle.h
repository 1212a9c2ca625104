/*
 * holo_oracle.h -- CPU FP64 restatement of the reference's Huygens superposition.
 *
 * TEST INFRASTRUCTURE ONLY.  This is the checker: tests, the smoke entry point
 * and the CPU-baseline leg of the benchmark call it.  The product path (the
 * CUDA library) never links or calls it.
 *
 * Every function cites the reference file:line it restates (paths relative to
 * the reference project root).
 */
#ifndef HOLO_ORACLE_H
#define HOLO_ORACLE_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* k = (2*pi)/lambda, evaluated as TWO_PI_OVER_LAMBDA is (cuda/macros.h:27-31). */
double oracle_wavenumber(double lambda);

/* One source/target term, cuda/superposition.cu:35-51 (phasor_displacement<dir>)
 * with norm3d_host (cuda/kernel.cu:95-99) and from_polar (cuda/kernel.cu:158-166).
 * sign = +1 is Direction::Forwards (phase + k r), -1 is Backwards (phase - k r).
 * out[0] = re, out[1] = im. */
void oracle_phasor(double amp, double phase, const double u[3], const double v[3],
                   int sign, double k, double out[2]);

/* Brute-force sum y_m = sum_n phasor(x_n, u_n, v_m) for every target, in source
 * order n = 0..N-1 (transform_full, cuda/transform.cu:147-340; the reference's
 * batching and cuBLAS row sum only change the order of the additions).
 * amp/phase: N doubles; u: N*3 xyz-interleaved; v: M*3; y: M*2 (re, im).
 * Uses up to nthreads host threads (<=0: 1).  Returns 0, or -1 on bad args. */
int oracle_transform(size_t N, const double *amp, const double *phase, const double *u,
                     size_t M, const double *v, int sign, double lambda,
                     double *y, int nthreads);

/* Same sum for a subset of targets: y_sub[2*i..] = y[idx[i]]. */
int oracle_transform_subset(size_t N, const double *amp, const double *phase, const double *u,
                            const double *v, const int64_t *idx, size_t n_idx,
                            int sign, double lambda, double *y_sub, int nthreads);

/* normalize_amp<false> (cuda/transform.cu:106-139): divide by max |y| unless
 * max |y| < 1e-6 (then unchanged).  Returns max |y| (cuCabs == hypot). */
double oracle_normalize_amp(double *y, size_t M);

/* Polar output (cuda/transform.cu:402-405): amp = |y|, phase = atan2(im, re). */
void oracle_to_polar(const double *y, size_t M, double *amp, double *phase);

/* Philox4x32-10 (Salmon, Moraes, Dror, Shaw: "Parallel random numbers: as easy
 * as 1, 2, 3", SC'11).  Counter-based generator used by the Monte Carlo
 * estimator; the CUDA side implements the same published rounds. */
void oracle_philox4x32_10(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4]);

/* Monte Carlo estimator with stratified source sampling.  The reference snapshot
 * has no MC code (only its RNG leftovers, cuda/kernel.cu:102-106, 197-212), so this
 * restates the estimator the library defines:
 *   sources in the order src_order[0..N-1] are cut into strata of `sub`
 *   consecutive entries; targets in the order tgt_order[0..M-1] are cut into
 *   blocks of `block` consecutive entries.  For target block b and stratum j,
 *   Philox4x32-10 with counter (j, b, 0, 0) and key (seed_lo, seed_hi) picks
 *   offset = out[0] mod size_j inside the stratum; the estimate for every target
 *   in block b is sum_j size_j * phasor(pick_j, target).
 * y is written in ORIGINAL target order. */
int oracle_transform_mc(size_t N, const double *amp, const double *phase, const double *u,
                        size_t M, const double *v, int sign, double lambda,
                        const int32_t *src_order, const int32_t *tgt_order,
                        uint64_t seed, int sub, int block,
                        double *y, int nthreads);

#ifdef __cplusplus
}
#endif
#endif
