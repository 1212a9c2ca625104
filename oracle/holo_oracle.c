/*
 * holo_oracle.c -- CPU FP64 restatement of the reference's Huygens superposition.
 *
 * TEST INFRASTRUCTURE ONLY (the checker; never part of the product path).
 * Build with -ffp-contract=off so that x86-64 and aarch64 round every product
 * and sum separately, exactly as written below.
 */
#include "holo_oracle.h"

#include <math.h>
#include <pthread.h>
#include <stdlib.h>
#include <string.h>

double oracle_wavenumber(double lambda) {
  /* TWO_PI_OVER_LAMBDA = (TWO_PI / LAMBDA), TWO_PI = (2 * M_PI): cuda/macros.h:27-31 */
  return (2.0 * M_PI) / lambda;
}

void oracle_phasor(double amp, double phase, const double u[3], const double v[3],
                   int sign, double k, double out[2]) {
  /* distance = NORM_3D(v[0]-u[0], v[1]-u[1], v[2]-u[2]) (cuda/superposition.cu:42);
   * norm3d_host is (a*a + b*b + c*c)^0.5 (cuda/kernel.cu:95-99).  sqrt is the
   * correctly rounded square root (pow(., 0.5) agrees with it to <= 1 ulp). */
  const double a = v[0] - u[0], b = v[1] - u[1], c = v[2] - u[2];
  const double s = a * a + b * b + c * c;
  const double distance = sqrt(s);
  /* Forwards: phase + distance * k, Backwards: phase - distance * k (superposition.cu:47-50) */
  const double kr = distance * k;
  const double next_phase = sign > 0 ? phase + kr : phase - kr;
  const double r = amp / distance;
  /* from_polar(r, phi) = {r cos phi, r sin phi} (cuda/kernel.cu:158-166) */
  out[0] = r * cos(next_phase);
  out[1] = r * sin(next_phase);
}

typedef struct {
  size_t N;
  const double *amp, *phase, *u, *v;
  const int64_t *idx; /* NULL: all targets */
  size_t m0, m1;
  int sign;
  double k;
  double *y;
} range_job;

static void *range_worker(void *arg) {
  const range_job *j = (const range_job *)arg;
  double t[2];
  for (size_t i = j->m0; i < j->m1; ++i) {
    const size_t m = j->idx ? (size_t)j->idx[i] : i;
    const double *vm = j->v + 3 * m;
    double re = 0.0, im = 0.0;
    for (size_t n = 0; n < j->N; ++n) {
      oracle_phasor(j->amp[n], j->phase[n], j->u + 3 * n, vm, j->sign, j->k, t);
      re += t[0];
      im += t[1];
    }
    j->y[2 * i] = re;
    j->y[2 * i + 1] = im;
  }
  return NULL;
}

static int run_ranges(size_t N, const double *amp, const double *phase, const double *u,
                      const double *v, const int64_t *idx, size_t count, int sign,
                      double lambda, double *y, int nthreads) {
  if (nthreads < 1) nthreads = 1;
  if ((size_t)nthreads > count) nthreads = count ? (int)count : 1;
  range_job *jobs = (range_job *)calloc((size_t)nthreads, sizeof(range_job));
  pthread_t *th = (pthread_t *)calloc((size_t)nthreads, sizeof(pthread_t));
  if (!jobs || !th) { free(jobs); free(th); return -1; }
  const double k = oracle_wavenumber(lambda);
  const size_t per = (count + (size_t)nthreads - 1) / (size_t)nthreads;
  int *joined = (int *)calloc((size_t)nthreads, sizeof(int));
  if (!joined) { free(jobs); free(th); return -1; }
  for (int t = 0; t < nthreads; ++t) {
    range_job *j = &jobs[t];
    j->N = N; j->amp = amp; j->phase = phase; j->u = u; j->v = v; j->idx = idx;
    j->m0 = (size_t)t * per < count ? (size_t)t * per : count;
    j->m1 = j->m0 + per < count ? j->m0 + per : count;
    j->sign = sign; j->k = k; j->y = y;
    if (t == 0) continue;
    if (pthread_create(&th[t], NULL, range_worker, j) == 0) joined[t] = 1;
    else range_worker(j); /* no thread available: run it here */
  }
  range_worker(&jobs[0]);
  for (int t = 1; t < nthreads; ++t)
    if (joined[t]) pthread_join(th[t], NULL);
  free(joined);
  free(jobs);
  free(th);
  return 0;
}

int oracle_transform(size_t N, const double *amp, const double *phase, const double *u,
                     size_t M, const double *v, int sign, double lambda,
                     double *y, int nthreads) {
  if ((N && (!amp || !phase || !u)) || (M && (!v || !y)) || lambda <= 0.0) return -1;
  return run_ranges(N, amp, phase, u, v, NULL, M, sign, lambda, y, nthreads);
}

int oracle_transform_subset(size_t N, const double *amp, const double *phase, const double *u,
                            const double *v, const int64_t *idx, size_t n_idx,
                            int sign, double lambda, double *y_sub, int nthreads) {
  if ((N && (!amp || !phase || !u)) || (n_idx && (!v || !idx || !y_sub)) || lambda <= 0.0)
    return -1;
  return run_ranges(N, amp, phase, u, v, idx, n_idx, sign, lambda, y_sub, nthreads);
}

double oracle_normalize_amp(double *y, size_t M) {
  /* cuda/transform.cu:106-139 with add_constant = false and to = 1 */
  double max_amp = 0.0;
  for (size_t i = 0; i < M; ++i) max_amp = fmax(max_amp, hypot(y[2 * i], y[2 * i + 1]));
  if (max_amp < 1e-6) return max_amp; /* "WARNING, max_amp << 1": left unnormalised */
  for (size_t i = 0; i < M; ++i) {
    y[2 * i] = y[2 * i] / max_amp;
    y[2 * i + 1] = y[2 * i + 1] / max_amp;
  }
  return max_amp;
}

void oracle_to_polar(const double *y, size_t M, double *amp, double *phase) {
  for (size_t i = 0; i < M; ++i) {
    amp[i] = hypot(y[2 * i], y[2 * i + 1]);
    phase[i] = atan2(y[2 * i + 1], y[2 * i]);
  }
}

/* ---- Philox4x32-10, published algorithm (SC'11), written from the paper ---- */
static inline void mulhilo32(uint32_t a, uint32_t b, uint32_t *hi, uint32_t *lo) {
  const uint64_t p = (uint64_t)a * (uint64_t)b;
  *hi = (uint32_t)(p >> 32);
  *lo = (uint32_t)p;
}

void oracle_philox4x32_10(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4]) {
  uint32_t c0 = ctr[0], c1 = ctr[1], c2 = ctr[2], c3 = ctr[3];
  uint32_t k0 = key[0], k1 = key[1];
  for (int round = 0; round < 10; ++round) {
    uint32_t hi0, lo0, hi1, lo1;
    mulhilo32(0xD2511F53u, c0, &hi0, &lo0);
    mulhilo32(0xCD9E8D57u, c2, &hi1, &lo1);
    const uint32_t n0 = hi1 ^ c1 ^ k0;
    const uint32_t n1 = lo1;
    const uint32_t n2 = hi0 ^ c3 ^ k1;
    const uint32_t n3 = lo0;
    c0 = n0; c1 = n1; c2 = n2; c3 = n3;
    k0 += 0x9E3779B9u;
    k1 += 0xBB67AE85u;
  }
  out[0] = c0; out[1] = c1; out[2] = c2; out[3] = c3;
}

typedef struct {
  size_t N, M;
  const double *amp, *phase, *u, *v;
  const int32_t *src_order, *tgt_order;
  uint64_t seed;
  int sub, block;
  size_t b0, b1; /* target blocks */
  int sign;
  double k;
  double *y;
} mc_job;

static void *mc_worker(void *arg) {
  const mc_job *j = (const mc_job *)arg;
  const size_t n_strata = (j->N + (size_t)j->sub - 1) / (size_t)j->sub;
  const uint32_t key[2] = {(uint32_t)j->seed, (uint32_t)(j->seed >> 32)};
  size_t *pick = (size_t *)malloc(n_strata * sizeof(size_t));
  double *w = (double *)malloc(n_strata * sizeof(double));
  double t[2];
  if (!pick || !w) { free(pick); free(w); return NULL; }
  for (size_t b = j->b0; b < j->b1; ++b) {
    for (size_t s = 0; s < n_strata; ++s) {
      const size_t start = s * (size_t)j->sub;
      const size_t size = (j->N - start) < (size_t)j->sub ? (j->N - start) : (size_t)j->sub;
      const uint32_t ctr[4] = {(uint32_t)s, (uint32_t)b, 0u, 0u};
      uint32_t out[4];
      oracle_philox4x32_10(ctr, key, out);
      pick[s] = (size_t)j->src_order[start + out[0] % (uint32_t)size];
      w[s] = (double)size;
    }
    const size_t t0 = b * (size_t)j->block;
    const size_t t1 = t0 + (size_t)j->block < j->M ? t0 + (size_t)j->block : j->M;
    for (size_t ti = t0; ti < t1; ++ti) {
      const size_t m = (size_t)j->tgt_order[ti];
      double re = 0.0, im = 0.0;
      for (size_t s = 0; s < n_strata; ++s) {
        const size_t n = pick[s];
        oracle_phasor(j->amp[n], j->phase[n], j->u + 3 * n, j->v + 3 * m, j->sign, j->k, t);
        re += w[s] * t[0];
        im += w[s] * t[1];
      }
      j->y[2 * m] = re;
      j->y[2 * m + 1] = im;
    }
  }
  free(pick);
  free(w);
  return NULL;
}

int oracle_transform_mc(size_t N, const double *amp, const double *phase, const double *u,
                        size_t M, const double *v, int sign, double lambda,
                        const int32_t *src_order, const int32_t *tgt_order,
                        uint64_t seed, int sub, int block,
                        double *y, int nthreads) {
  if (sub < 1 || block < 1 || lambda <= 0.0) return -1;
  if ((N && (!amp || !phase || !u || !src_order)) || (M && (!v || !y || !tgt_order))) return -1;
  if (N == 0) {
    memset(y, 0, 2 * M * sizeof(double));
    return 0;
  }
  const size_t n_blocks = (M + (size_t)block - 1) / (size_t)block;
  if (nthreads < 1) nthreads = 1;
  if ((size_t)nthreads > n_blocks) nthreads = n_blocks ? (int)n_blocks : 1;
  mc_job *jobs = (mc_job *)calloc((size_t)nthreads, sizeof(mc_job));
  pthread_t *th = (pthread_t *)calloc((size_t)nthreads, sizeof(pthread_t));
  if (!jobs || !th) { free(jobs); free(th); return -1; }
  const size_t per = (n_blocks + (size_t)nthreads - 1) / (size_t)nthreads;
  int *joined = (int *)calloc((size_t)nthreads, sizeof(int));
  if (!joined) { free(jobs); free(th); return -1; }
  for (int t = 0; t < nthreads; ++t) {
    mc_job *j = &jobs[t];
    j->N = N; j->M = M; j->amp = amp; j->phase = phase; j->u = u; j->v = v;
    j->src_order = src_order; j->tgt_order = tgt_order;
    j->seed = seed; j->sub = sub; j->block = block;
    j->b0 = (size_t)t * per < n_blocks ? (size_t)t * per : n_blocks;
    j->b1 = j->b0 + per < n_blocks ? j->b0 + per : n_blocks;
    j->sign = sign; j->k = oracle_wavenumber(lambda); j->y = y;
    if (t == 0) continue;
    if (pthread_create(&th[t], NULL, mc_worker, j) == 0) joined[t] = 1;
    else mc_worker(j);
  }
  mc_worker(&jobs[0]);
  for (int t = 1; t < nthreads; ++t)
    if (joined[t]) pthread_join(th[t], NULL);
  free(joined);
  free(jobs);
  free(th);
  return 0;
}
