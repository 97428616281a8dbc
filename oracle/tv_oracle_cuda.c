/*
 * tv_oracle_cuda.c -- CPU restatement of the reference's CUDA backend.
 *
 * TEST INFRASTRUCTURE ONLY.  It states, in plain C with IEEE double
 * arithmetic, the values the reference's CUDA kernels (src/kernels.cu, driven
 * by src/hsmm.cu:604-791) compute, so that their results on the GPU can be
 * checked and every place where they differ from the reference's C++ decoder
 * (src/hsmm.cu:233-373, restated in tv_oracle.c) can be named.  Four
 * differences, each switchable with a flag bit; with no bit set this is the
 * C++ decoder again (checked against tv_oracle.c by the tests):
 *
 *   TVO_CU_INIT_SCAN  the initial scores delta[t<D][j] = (dur + start) + E,
 *                     with E the emission prefix sum in kernel_initialization's
 *                     block-scan association (src/kernels.cu:94-127): warp
 *                     Hillis-Steele scans, a scan of the warp totals, and a
 *                     running offset per block-sized chunk; the C++ decoder
 *                     sums oldest-first (src/hsmm.cu:274-290).
 *   TVO_CU_WINDOW     the emission window rolled from t = 1,
 *                     E_t[d] = em_t + E_{t-1}[d-1] (src/kernels.cu:163-175);
 *                     the C++ decoder rebuilds it newest-first for t <= D
 *                     (src/hsmm.cu:311-328) and rolls only after.
 *   TVO_CU_TAIL       the tail score (E + delta) + (trans + log S), with S the
 *                     linear duration suffix sum in the same block-scan
 *                     association (src/kernels.cu:43-78, 448-458); the C++
 *                     decoder uses ((E + logsurv) + delta) + trans with a
 *                     log-space survival (src/hsmm.cu:79-137).
 *   TVO_CU_ITREE      the argmax: per (j, i) the best d (lowest d on ties), then
 *                     kernel_reduce_i's tree over i (src/kernels.cu:228-300),
 *                     strict '>' between tree slots, so a tie across i is not
 *                     always won by the lowest i nor by the lowest d; the C++
 *                     decoder takes the lowest (d, i), d outer (:335-359).
 *
 * The device's log may differ from the C library's in the last place; the
 * tail can take the device's values of log S (log_suffix) instead.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#include "tv_oracle.h"

#define DUR(d, j) duration[(size_t)(d) * N + (j)]
#define EMI(o, j) emission[(size_t)(o) * N + (j)]

static int pow2_at_least(int x) {
    int p = 1;
    while (p < x) p <<= 1;
    return p;
}

/* One Hillis-Steele inclusive scan per warp over the lanes [0, w): lane k
 * adds the value `stride` lanes below it (__shfl_up_sync) at strides
 * 1, 2, 4, 8, 16, all lanes at once. */
static void warp_scan(double* v, int w) {
    double old[32];
    for (int stride = 1; stride < 32; stride <<= 1) {
        memcpy(old, v, sizeof(double) * (size_t)w);
        for (int k = stride; k < w; ++k) v[k] = old[k] + old[k - stride];
    }
}

/* Inclusive prefix sums of x[0..n) in kernel_initialization's association,
 * for a block of bs = min(next_pow2(n), 1024) threads (src/kernels.cu:43-78
 * and :94-127). */
void tvo_block_scan(const double* x, int n, double* out) {
    int bs = pow2_at_least(n);
    if (bs > 1024) bs = 1024;
    const int nw = bs / 32;
    double* v = (double*)malloc(sizeof(double) * (size_t)bs);
    double ws[32];
    double running = 0.0;
    for (int base = 0; base < n; base += bs) {
        for (int k = 0; k < bs; ++k) v[k] = (base + k < n) ? x[base + k] : 0.0;
        const int lanes = bs < 32 ? bs : 32;
        for (int w0 = 0; w0 < bs; w0 += lanes) warp_scan(v + w0, lanes);
        /* warp totals (lane 31 of each warp), scanned by the first warp */
        for (int d = 0; d < 32; ++d) ws[d] = d < nw ? v[32 * d + 31] : 0.0;
        warp_scan(ws, 32);
        for (int k = 0; k < bs && base + k < n; ++k) {
            const int w = k / 32;
            out[base + k] = (w > 0 ? v[k] + ws[w - 1] : v[k]) + running;
        }
        /* the chunk total: the last warp total, or, for a block below one
         * warp (no warp total is written), the slot just below the totals,
         * which is the last scanned value */
        running += nw > 0 ? ws[nw - 1] : v[bs - 1];
    }
    free(v);
}

/* Linear duration suffix sums as kernel_initialization forms them:
 * out[j*D + d] = the block scan of lin[D-1..0][j] at position D-1-d. */
void tvo_lin_suffix(int N, int D, const double* dur_lin, double* out) {
    double* x = (double*)malloc(sizeof(double) * (size_t)D);
    double* s = (double*)malloc(sizeof(double) * (size_t)D);
    for (int j = 0; j < N; ++j) {
        for (int k = 0; k < D; ++k) x[k] = dur_lin[(size_t)(D - 1 - k) * N + j];
        tvo_block_scan(x, D, s);
        for (int d = 0; d < D; ++d) out[(size_t)j * D + d] = s[D - 1 - d];
    }
    free(x);
    free(s);
}

/* kernel_reduce_i's tree over the per-i winners (val[i], dd[i]): slots padded
 * to next_pow2(N) with -1e300, halving strides down to one warp, then the
 * warp's shuffle-down halving; strict '>' keeps the left slot on a tie. */
static void reduce_i_tree(int N, const double* val, const int* dd, double* bv, int* bi, int* bd,
                          double* sv, int* si, int* sd) {
    const int bs = pow2_at_least(N);
    for (int i = 0; i < bs; ++i) {
        sv[i] = i < N ? val[i] : -1e300;
        si[i] = i < N ? i : 0;
        sd[i] = i < N ? dd[i] : 0;
    }
    for (int stride = bs >> 1; stride >= 32; stride >>= 1)
        for (int i = 0; i < stride; ++i)
            if (sv[i + stride] > sv[i]) { sv[i] = sv[i + stride]; si[i] = si[i + stride]; sd[i] = sd[i + stride]; }
    const int w = bs < 32 ? bs : 32;
    for (int stride = (bs >> 1) < 16 ? (bs >> 1) : 16; stride > 0; stride >>= 1)
        for (int lane = 0; lane + stride < w; ++lane)  /* lanes in increasing order read higher, not yet updated, lanes */
            if (sv[lane + stride] > sv[lane]) { sv[lane] = sv[lane + stride]; si[lane] = si[lane + stride]; sd[lane] = sd[lane + stride]; }
    *bv = sv[0];
    *bi = si[0];
    *bd = sd[0];
}

/* Best candidate for state j at one step.  cand(d, i) gives the score; the
 * C++ rule takes the lowest (d, i) with d outer, the CUDA rule the per-i
 * lowest d and then the tree over i. */
typedef struct {
    int N, tau, itree;
    const double* w;     /* window value per d (this state) */
    const double* add;   /* second term per d: dur (induction) or unused */
    const double* delta; /* time-major T x N */
    const double* trans; /* row j */
    const double* tailw; /* per d: C++ tail: E + logsurv ; CUDA tail: unused */
    const double* logs;  /* per d: CUDA tail: log S (row j) */
    int t, mode;         /* mode 0 induction, 1 C++ tail, 2 CUDA tail */
} Step;

static inline double cand(const Step* s, int d, int i) {
    const double prev = s->delta[(size_t)(s->t - 1 - d) * s->N + i];
    switch (s->mode) {
        case 0: return (s->w[d] + prev) + (s->trans[i] + s->add[d]);
        case 1: return (s->tailw[d] + prev) + s->trans[i];
        default: return (s->w[d] + prev) + (s->trans[i] + s->logs[d]);
    }
}

static void best_of(const Step* s, double* bv, int* bi, int* bd, double* vi, int* di, double* sv, int* si, int* sd) {
    if (!s->itree) {
        double best = -INFINITY;
        int b_d = 0, b_i = 0;
        for (int d = 0; d < s->tau; ++d)
            for (int i = 0; i < s->N; ++i) {
                const double v = cand(s, d, i);
                if (v > best) { best = v; b_d = d; b_i = i; }
            }
        *bv = best; *bi = b_i; *bd = b_d;
        return;
    }
    for (int i = 0; i < s->N; ++i) {
        double val = -1e300;
        int dd = 0;
        for (int d = 0; d < s->tau; ++d) {
            const double v = cand(s, d, i);
            if (v > val || (v == val && d < dd)) { val = v; dd = d; }
        }
        vi[i] = val;
        di[i] = dd;
    }
    reduce_i_tree(s->N, vi, di, bv, bi, bd, sv, si, sd);
}

/*
 * Decode with the selected CUDA-backend semantics (flags) and the C++
 * decoder's rules elsewhere.  Layouts as tvo_decode; dur_lin (D,N) linear.
 * log_suffix (N x D, [j][d]) may be NULL: the tail then takes the C
 * library's log of tvo_lin_suffix.  final (N) may be NULL.
 */
int tvo_decode_cuda(int N, int O, int D, int T, const double* trans, const double* emission,
                    const double* dur_lin, const double* start, const double* duration, const int32_t* obs,
                    int flags, const double* log_suffix, int nthreads, int32_t* path, double* loglik,
                    double* final) {
    int rc = tvo_check_args(N, O, D, T, obs);
    if (rc != TVO_OK) return rc;
    const int bsN = pow2_at_least(N);
    double* delta = (double*)malloc(sizeof(double) * (size_t)T * N);
    int32_t* ps = (int32_t*)calloc((size_t)T * N, sizeof(int32_t));
    int32_t* pd = (int32_t*)malloc(sizeof(int32_t) * (size_t)T * N);
    double* win = (double*)malloc(sizeof(double) * (size_t)D * N);  /* [j][d] */
    double* nwin = (double*)malloc(sizeof(double) * (size_t)D * N);
    double* surv = (double*)malloc(sizeof(double) * (size_t)D * N); /* C++: [d][j] */
    double* logs = (double*)malloc(sizeof(double) * (size_t)D * N); /* CUDA: [j][d] */
    double* durT = (double*)malloc(sizeof(double) * (size_t)D * N); /* [j][d] */
    double* x = (double*)malloc(sizeof(double) * (size_t)D);
    double* e = (double*)malloc(sizeof(double) * (size_t)D);
    if (!delta || !ps || !pd || !win || !nwin || !surv || !logs || !durT || !x || !e) {
        rc = TVO_ENOMEM;
        goto out;
    }
    for (int j = 0; j < N; ++j)
        for (int d = 0; d < D; ++d) durT[(size_t)j * D + d] = DUR(d, j);
    tvo_survival(N, D, duration, surv);
    if (log_suffix) {
        memcpy(logs, log_suffix, sizeof(double) * (size_t)D * N);
    } else {
        tvo_lin_suffix(N, D, dur_lin, logs);
        for (size_t k = 0; k < (size_t)D * N; ++k) logs[k] = log(logs[k]);
    }

    /* initialisation, t < D */
    for (int j = 0; j < N; ++j) {
        for (int d = 0; d < D; ++d) x[d] = EMI(obs[d], j);
        if (flags & TVO_CU_INIT_SCAN) {
            tvo_block_scan(x, D, e);
        } else {
            double acc = 0.0;
            for (int d = 0; d < D; ++d) { acc = acc + x[d]; e[d] = acc; }
        }
        for (int d = 0; d < D; ++d) {
            delta[(size_t)d * N + j] = (DUR(d, j) + start[j]) + e[d];
            pd[(size_t)d * N + j] = d + 1;
        }
    }

#ifdef _OPENMP
    if (nthreads > 0) omp_set_num_threads(nthreads);
#else
    (void)nthreads;
#endif
    for (int t = 1; t < T; ++t) {
        const int tau = t < D ? t : D;
        const int ot = obs[t];
        /* the window at step t, [j][d] for d < tau */
        for (int j = 0; j < N; ++j) {
            double* wj = win + (size_t)j * D;
            double* nj = nwin + (size_t)j * D;
            const double em = EMI(ot, j);
            if ((flags & TVO_CU_WINDOW) || t > D) {
                nj[0] = em;
                for (int d = 1; d < tau; ++d) nj[d] = em + wj[d - 1];
            } else {
                nj[0] = em;
                for (int d = 1; d < tau; ++d) nj[d] = nj[d - 1] + EMI(obs[t - d], j);
            }
        }
        { double* tmp = win; win = nwin; nwin = tmp; }
        #pragma omp parallel
        {
            double* vi = (double*)malloc(sizeof(double) * (size_t)N);
            int* di = (int*)malloc(sizeof(int) * (size_t)N);
            double* sv = (double*)malloc(sizeof(double) * (size_t)bsN);
            int* si = (int*)malloc(sizeof(int) * (size_t)bsN);
            int* sd = (int*)malloc(sizeof(int) * (size_t)bsN);
            #pragma omp for schedule(static)
            for (int j = 0; j < N; ++j) {
                Step s = {N, tau, (flags & TVO_CU_ITREE) != 0, win + (size_t)j * D, durT + (size_t)j * D, delta,
                          trans + (size_t)j * N, NULL, NULL, t, 0};
                double bv;
                int bi, bd;
                best_of(&s, &bv, &bi, &bd, vi, di, sv, si, sd);
                double* slot = delta + (size_t)t * N + j;
                if (t >= D || bv > *slot) {
                    *slot = bv;
                    ps[(size_t)t * N + j] = bi;
                    pd[(size_t)t * N + j] = bd + 1;
                }
            }
            free(vi); free(di); free(sv); free(si); free(sd);
        }
    }

    /* tail at t = T-1: unconditional overwrite */
    {
        const int t = T - 1;
        const int tau = t < D ? t : D;
        double* tl = (double*)malloc(sizeof(double) * (size_t)N);
        double* vi = (double*)malloc(sizeof(double) * (size_t)N);
        int* di = (int*)malloc(sizeof(int) * (size_t)N);
        double* sv = (double*)malloc(sizeof(double) * (size_t)bsN);
        int* si = (int*)malloc(sizeof(int) * (size_t)bsN);
        int* sd = (int*)malloc(sizeof(int) * (size_t)bsN);
        if (!tl || !vi || !di || !sv || !si || !sd) {
            free(tl); free(vi); free(di); free(sv); free(si); free(sd);
            rc = TVO_ENOMEM;
            goto out;
        }
        for (int j = 0; j < N; ++j) {
            for (int d = 0; d < tau; ++d) x[d] = win[(size_t)j * D + d] + surv[(size_t)d * N + j];
            Step s = {N, tau, (flags & TVO_CU_ITREE) != 0, win + (size_t)j * D, NULL, delta, trans + (size_t)j * N,
                      x, logs + (size_t)j * D, t, (flags & TVO_CU_TAIL) ? 2 : 1};
            double bv;
            int bi, bd;
            best_of(&s, &bv, &bi, &bd, vi, di, sv, si, sd);
            tl[j] = bv;
            ps[(size_t)t * N + j] = bi;
            pd[(size_t)t * N + j] = bd + 1;
        }
        /* backtrace (src/hsmm.cu:139-170) */
        int cur = 0;
        double best = tl[0];
        for (int n = 1; n < N; ++n)
            if (tl[n] > best) { best = tl[n]; cur = n; }
        if (final) memcpy(final, tl, sizeof(double) * (size_t)N);
        if (loglik) *loglik = best;
        int tt = T - 1;
        while (tt >= 0) {
            const int len = pd[(size_t)tt * N + cur];
            const int prev = ps[(size_t)tt * N + cur];
            for (int k = tt - len + 1; k <= tt; ++k) path[k] = cur;
            tt -= len;
            cur = prev;
        }
        free(tl); free(vi); free(di); free(sv); free(si); free(sd);
    }
out:
    free(delta); free(ps); free(pd); free(win); free(nwin); free(surv); free(logs); free(durT); free(x); free(e);
    return rc;
}
