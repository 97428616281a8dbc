/*
 * tv_oracle.c -- CPU restatement of the reference HSMM tensor-Viterbi decoder.
 *
 * TEST INFRASTRUCTURE ONLY.  This file is the checker for the GPU decoder and
 * the CPU baseline that bench.py times beside it.  No product code path may
 * link, load or call it.
 *
 * It restates, in plain C with IEEE double arithmetic, the semantics of the
 * reference project's CPU decoders:
 *   serial  decode_tensor_viterbi      src/hsmm.cu:233-373
 *   OpenMP  decode_tensor_viterbi_omp  src/hsmm.cu:376-600
 *   helpers compute_survival_probs     src/hsmm.cu:79-99
 *           tail_adjustment            src/hsmm.cu:101-137
 *           backtracking_termination   src/hsmm.cu:139-170
 * Every floating-point expression keeps the reference's association, so the
 * score tables (delta, psi) match the reference bit for bit when both are
 * compiled without -ffast-math.
 *
 * Input layout is the Python-facing one of the reference binding
 * (src/bindings.cpp:19-56): trans (N,N) indexed [to j][from i], emission
 * (O,N), start (N), duration (D,N); all log space.  obs is 0-based int32.
 *
 * Pinning: tests/golden/make_golden.py runs the reference's own compiled
 * `_native` module (oracle/build_ref.sh) on the reference's data fixtures and
 * on seeded synthetic models and stores its paths; tests/test_oracle.py checks
 * this file against those paths.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#include "tv_oracle.h"

#define NEG_INF (-INFINITY)

/* Index helpers for the Python (D,N) / (O,N) layouts. */
#define DUR(d, j) duration[(size_t)(d) * N + (j)]
#define EMI(o, j) emission[(size_t)(o) * N + (j)]

int tvo_check_args(int N, int O, int D, int T, const int32_t* obs) {
    if (N <= 0 || O <= 0 || D <= 0 || T <= 0) return TVO_EINVAL;
    /* The reference initialisation reads obs[0..D) and writes D rows of the
     * T-row score table (src/hsmm.cu:276-290), so it needs T >= D. */
    if (T < D) return TVO_ESHORT;
    for (int t = 0; t < T; ++t)
        if (obs[t] < 0 || obs[t] >= O) return TVO_ERANGE;
    return TVO_OK;
}

/* Log-space survival table surv[d*N + j] = log sum_{d' >= d} exp(dur[d'][j]),
 * accumulated from d = D-1 downwards with the running two-term log-sum-exp of
 * src/hsmm.cu:79-99. */
void tvo_survival(int N, int D, const double* duration, double* surv) {
    for (int j = 0; j < N; ++j) {
        double acc = NEG_INF;
        for (int d = D - 1; d >= 0; --d) {
            const double lp = DUR(d, j);
            const double hi = (acc < lp) ? lp : acc; /* std::max(acc, lp) */
            if (hi == NEG_INF)
                acc = lp;
            else
                acc = hi + log(exp(acc - hi) + exp(lp - hi));
            surv[(size_t)d * N + j] = acc;
        }
    }
}

/* Follows (psi_dur, psi_state) back from the best final state
 * (src/hsmm.cu:139-170).  psi arrays are time-major [t*N + j] here.
 * final_score[j] holds the tail-adjusted scores at t = T-1. */
static double backtrace(int N, int T, const double* final_score,
                        const int32_t* psi_state, const int32_t* psi_dur,
                        int32_t* path, uint8_t* seg_start) {
    int cur = 0;
    double best = final_score[0];
    for (int n = 1; n < N; ++n)
        if (final_score[n] > best) { best = final_score[n]; cur = n; }
    if (seg_start) memset(seg_start, 0, (size_t)T);
    int t = T - 1;
    while (t >= 0) {
        const int len = psi_dur[(size_t)t * N + cur];
        const int prev = psi_state[(size_t)t * N + cur];
        const int first = t - len + 1;
        for (int k = first; k <= t; ++k) path[k] = cur;
        if (seg_start) seg_start[first] = 1;
        t -= len;
        cur = prev;
    }
    return best;
}

/* ------------------------------------------------------------------------ */
/* Serial decoder: src/hsmm.cu:233-373.                                      */
/* ------------------------------------------------------------------------ */
static int decode_serial(int N, int O, int D, int T,
                         const double* trans, const double* emission,
                         const double* start, const double* duration,
                         const int32_t* obs, const double* surv,
                         double* delta_t, int32_t* psi_state, int32_t* psi_dur,
                         double* tail) {
    (void)O;
    double* win = (double*)malloc(sizeof(double) * (size_t)D * N);   /* EMISSION_PROBS */
    double* shift = (double*)calloc((size_t)D * N, sizeof(double));  /* EMISSION_CACHE */
    if (!win || !shift) { free(win); free(shift); return TVO_ENOMEM; }

    /* Initialisation, t < D: a single segment [0, t] of state j
     * (src/hsmm.cu:274-290).  win[d] is the oldest-first running sum. */
    for (int d = 0; d < D; ++d)
        for (int j = 0; j < N; ++j) {
            const double before = d > 0 ? win[(size_t)(d - 1) * N + j] : 0.0;
            win[(size_t)d * N + j] = before + EMI(obs[d], j);
        }
    for (int d = 0; d < D; ++d)
        for (int j = 0; j < N; ++j) {
            delta_t[(size_t)d * N + j] = (DUR(d, j) + start[j]) + win[(size_t)d * N + j];
            psi_dur[(size_t)d * N + j] = d + 1;
        }

    /* Induction (src/hsmm.cu:292-360). */
    for (int t = 1; t < T; ++t) {
        const int tau = t < D ? t : D;
        const int ot = obs[t];
        if (t > D) {
            /* win_t[d] = win_{t-1}[d-1] + em_t, with win_t[0] = 0 + em_t:
             * the rolling update through the shift buffer (:298-310). */
            for (int d = 0; d < D; ++d)
                for (int j = 0; j < N; ++j)
                    win[(size_t)d * N + j] = shift[(size_t)d * N + j] + EMI(ot, j);
            memcpy(shift + N, win, sizeof(double) * (size_t)(D - 1) * N);
        } else {
            /* Rebuilt newest-first for t <= D (:311-328). */
            for (int j = 0; j < N; ++j) win[j] = EMI(ot, j);
            for (int d = 1; d < tau; ++d)
                for (int j = 0; j < N; ++j)
                    win[(size_t)d * N + j] = win[(size_t)(d - 1) * N + j] + EMI(obs[t - d], j);
            if (t == D) memcpy(shift + N, win, sizeof(double) * (size_t)(D - 1) * N);
        }
        /* Joint argmax over (d, i), d outer and i inner, strict '>' from -inf:
         * the lowest d, then the lowest i, wins a tie (:335-359). */
        for (int j = 0; j < N; ++j) {
            double best = NEG_INF;
            int bd = 0, bi = 0;
            for (int d = 0; d < tau; ++d) {
                const double w = win[(size_t)d * N + j];
                const double dj = DUR(d, j);
                const double* prev = delta_t + (size_t)(t - 1 - d) * N;
                const double* tr = trans + (size_t)j * N;
                for (int i = 0; i < N; ++i) {
                    const double v = (w + prev[i]) + (tr[i] + dj);
                    if (v > best) { best = v; bd = d; bi = i; }
                }
            }
            double* slot = delta_t + (size_t)t * N + j;
            if (t >= D || best > *slot) {
                *slot = best;
                psi_state[(size_t)t * N + j] = bi;
                psi_dur[(size_t)t * N + j] = bd + 1;
            }
        }
    }

    /* Tail adjustment at t = T-1 with survival in place of the duration pmf;
     * unconditional overwrite (src/hsmm.cu:101-137). */
    {
        const int t = T - 1;
        const int tau = t < D ? t : D;
        for (int j = 0; j < N; ++j) {
            double best = NEG_INF;
            int bd = 0, bi = 0;
            for (int d = 0; d < tau; ++d) {
                const double e = win[(size_t)d * N + j] + surv[(size_t)d * N + j];
                const double* prev = delta_t + (size_t)(t - 1 - d) * N;
                const double* tr = trans + (size_t)j * N;
                for (int i = 0; i < N; ++i) {
                    const double v = (e + prev[i]) + tr[i];
                    if (v > best) { best = v; bd = d; bi = i; }
                }
            }
            tail[j] = best;
            psi_state[(size_t)t * N + j] = bi;
            psi_dur[(size_t)t * N + j] = bd + 1;
        }
    }
    free(win);
    free(shift);
    return TVO_OK;
}

/* ------------------------------------------------------------------------ */
/* OpenMP decoder: src/hsmm.cu:376-600.  One parallel region; per step an    */
/* emission update, a per-(j,d) best-over-i pass and a per-j best-over-d     */
/* pass, separated by the implicit barriers of the work-sharing loops.  The  */
/* per-element arithmetic is the serial decoder's, so the tables are equal.  */
/* ------------------------------------------------------------------------ */
static int decode_openmp(int N, int O, int D, int T,
                         const double* trans, const double* emission,
                         const double* start, const double* duration,
                         const int32_t* obs, const double* surv,
                         double* delta_t, int32_t* psi_state, int32_t* psi_dur,
                         double* tail, int nthreads) {
    (void)O;
    const size_t ND = (size_t)N * D;
    double* win = (double*)malloc(sizeof(double) * ND);
    double* shift = (double*)calloc(ND, sizeof(double));
    double* part_v = (double*)malloc(sizeof(double) * ND);  /* best over i per (j,d) */
    int32_t* part_i = (int32_t*)malloc(sizeof(int32_t) * ND);
    if (!win || !shift || !part_v || !part_i) {
        free(win); free(shift); free(part_v); free(part_i);
        return TVO_ENOMEM;
    }
#ifdef _OPENMP
    if (nthreads <= 0) nthreads = omp_get_max_threads();
#else
    (void)nthreads;
#endif

#pragma omp parallel num_threads(nthreads) default(shared)
    {
#pragma omp for schedule(static)
        for (int j = 0; j < N; ++j) {
            double run = 0.0;
            for (int d = 0; d < D; ++d) {
                run += EMI(obs[d], j);
                win[(size_t)d * N + j] = run;
            }
        }
#pragma omp for schedule(static) collapse(2)
        for (int d = 0; d < D; ++d)
            for (int j = 0; j < N; ++j) {
                delta_t[(size_t)d * N + j] = (DUR(d, j) + start[j]) + win[(size_t)d * N + j];
                psi_dur[(size_t)d * N + j] = d + 1;
            }

        for (int t = 1; t < T; ++t) {
            const int tau = t < D ? t : D;
            const int ot = obs[t];
            if (t > D) {
#pragma omp for schedule(static) collapse(2)
                for (int d = 0; d < D; ++d)
                    for (int j = 0; j < N; ++j)
                        win[(size_t)d * N + j] = shift[(size_t)d * N + j] + EMI(ot, j);
#pragma omp for schedule(static)
                for (size_t k = 0; k < (size_t)(D - 1) * N; ++k) shift[N + k] = win[k];
            } else {
#pragma omp for schedule(static)
                for (int j = 0; j < N; ++j) {
                    win[j] = EMI(ot, j);
                    for (int d = 1; d < tau; ++d)
                        win[(size_t)d * N + j] = win[(size_t)(d - 1) * N + j] + EMI(obs[t - d], j);
                }
                if (t == D) {
#pragma omp for schedule(static)
                    for (size_t k = 0; k < (size_t)(D - 1) * N; ++k) shift[N + k] = win[k];
                }
            }
#pragma omp for schedule(static) collapse(2)
            for (int j = 0; j < N; ++j)
                for (int d = 0; d < tau; ++d) {
                    const double w = win[(size_t)d * N + j];
                    const double dj = DUR(d, j);
                    const double* prev = delta_t + (size_t)(t - 1 - d) * N;
                    const double* tr = trans + (size_t)j * N;
                    double best = NEG_INF;
                    int bi = 0;
                    for (int i = 0; i < N; ++i) {
                        const double v = (w + prev[i]) + (tr[i] + dj);
                        if (v > best) { best = v; bi = i; }
                    }
                    part_v[(size_t)j * D + d] = best;
                    part_i[(size_t)j * D + d] = bi;
                }
#pragma omp for schedule(static)
            for (int j = 0; j < N; ++j) {
                double best = NEG_INF;
                int bd = 0, bi = 0;
                for (int d = 0; d < tau; ++d)
                    if (part_v[(size_t)j * D + d] > best) {
                        best = part_v[(size_t)j * D + d];
                        bd = d;
                        bi = part_i[(size_t)j * D + d];
                    }
                double* slot = delta_t + (size_t)t * N + j;
                if (t >= D || best > *slot) {
                    *slot = best;
                    psi_state[(size_t)t * N + j] = bi;
                    psi_dur[(size_t)t * N + j] = bd + 1;
                }
            }
        }

        {
            const int t = T - 1;
            const int tau = t < D ? t : D;
#pragma omp for schedule(static) collapse(2)
            for (int j = 0; j < N; ++j)
                for (int d = 0; d < tau; ++d) {
                    const double e = win[(size_t)d * N + j] + surv[(size_t)d * N + j];
                    const double* prev = delta_t + (size_t)(t - 1 - d) * N;
                    const double* tr = trans + (size_t)j * N;
                    double best = NEG_INF;
                    int bi = 0;
                    for (int i = 0; i < N; ++i) {
                        const double v = (e + prev[i]) + tr[i];
                        if (v > best) { best = v; bi = i; }
                    }
                    part_v[(size_t)j * D + d] = best;
                    part_i[(size_t)j * D + d] = bi;
                }
#pragma omp for schedule(static)
            for (int j = 0; j < N; ++j) {
                double best = NEG_INF;
                int bd = 0, bi = 0;
                for (int d = 0; d < tau; ++d)
                    if (part_v[(size_t)j * D + d] > best) {
                        best = part_v[(size_t)j * D + d];
                        bd = d;
                        bi = part_i[(size_t)j * D + d];
                    }
                tail[j] = best;
                psi_state[(size_t)t * N + j] = bi;
                psi_dur[(size_t)t * N + j] = bd + 1;
            }
        }
    }
    free(win); free(shift); free(part_v); free(part_i);
    return TVO_OK;
}

int tvo_decode(int N, int O, int D, int T,
               const double* trans, const double* emission,
               const double* start, const double* duration,
               const int32_t* obs, int variant, int nthreads,
               int32_t* path_out, double* loglik_out,
               double* delta_out, double* tail_out,
               int32_t* psi_state_out, int32_t* psi_dur_out,
               uint8_t* seg_start_out) {
    int rc = tvo_check_args(N, O, D, T, obs);
    if (rc != TVO_OK) return rc;
    const size_t TN = (size_t)T * N;
    double* delta_t = delta_out ? delta_out : (double*)malloc(sizeof(double) * TN);
    int32_t* ps = psi_state_out ? psi_state_out : (int32_t*)malloc(sizeof(int32_t) * TN);
    int32_t* pd = psi_dur_out ? psi_dur_out : (int32_t*)malloc(sizeof(int32_t) * TN);
    double* surv = (double*)malloc(sizeof(double) * (size_t)D * N);
    double* tail = (double*)malloc(sizeof(double) * (size_t)N);
    if (!delta_t || !ps || !pd || !surv || !tail) { rc = TVO_ENOMEM; goto out; }
    for (size_t k = 0; k < TN; ++k) { delta_t[k] = NEG_INF; ps[k] = 0; pd[k] = 1; }
    tvo_survival(N, D, duration, surv);
    if (variant == 1)
        rc = decode_openmp(N, O, D, T, trans, emission, start, duration, obs, surv,
                           delta_t, ps, pd, tail, nthreads);
    else
        rc = decode_serial(N, O, D, T, trans, emission, start, duration, obs, surv,
                           delta_t, ps, pd, tail);
    if (rc != TVO_OK) goto out;
    {
        const double best = backtrace(N, T, tail, ps, pd, path_out, seg_start_out);
        if (loglik_out) *loglik_out = best;
        if (tail_out) memcpy(tail_out, tail, sizeof(double) * (size_t)N);
    }
out:
    if (!delta_out) free(delta_t);
    if (!psi_state_out) free(ps);
    if (!psi_dur_out) free(pd);
    free(surv);
    free(tail);
    return rc;
}

/* Independent scorer of a decoded segmentation, for the log-likelihood check.
 * Term for term it is the score the recursion assigns to that segmentation:
 * the first segment [0, e] takes start + dur[e] + sum of its emissions
 * (initialisation, src/hsmm.cu:283-290); every later segment takes
 * trans[to][from] + dur[len-1] + its emissions (induction, :341-346), and the
 * last segment takes the survival value in place of dur (:119-129).
 * Summed in long double, so its own rounding is far below the 1e-9 check. */
double tvo_score_segments(int N, int O, int D, int T,
                          const double* trans, const double* emission,
                          const double* start, const double* duration,
                          const int32_t* obs, const int32_t* path,
                          const uint8_t* seg_start) {
    (void)O;
    if (T <= 0) return NAN;
    double* surv = (double*)malloc(sizeof(double) * (size_t)D * N);
    if (!surv) return NAN;
    tvo_survival(N, D, duration, surv);
    long double total = 0.0L;
    int first = 1;
    int prev_state = -1;
    int t = 0;
    while (t < T) {
        int e = t;
        while (e + 1 < T && !seg_start[e + 1]) ++e;
        const int j = path[t];
        const int len = e - t + 1;
        if (len > D) { free(surv); return NAN; }
        long double em = 0.0L;
        for (int k = t; k <= e; ++k) em += EMI(obs[k], j);
        long double seg;
        const int last = (e == T - 1);
        if (first) {
            seg = (long double)start[j] + DUR(len - 1, j);
        } else {
            const long double tr = trans[(size_t)j * N + prev_state];
            seg = tr + (last ? surv[(size_t)(len - 1) * N + j] : DUR(len - 1, j));
        }
        total += seg + em;
        first = 0;
        prev_state = j;
        t = e + 1;
    }
    free(surv);
    return (double)total;
}
