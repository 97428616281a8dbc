/*
 * ref_cuda.c -- host driver for the reference project's own CUDA kernels.
 *
 * TEST INFRASTRUCTURE ONLY (parity and timing of the reference CUDA backend on
 * this GPU); no product code path links, loads or calls it.
 *
 * The kernels are the reference's: src/kernels.cu compiled for sm_103a with
 * the reference's CUDA flags into oracle/_ref/cuda/kernels_sm103a.cubin by
 * oracle/build_ref.sh (device code only, so the same file serves the x86 and
 * the aarch64 host).  This file restates, with the CUDA driver API, the host
 * side that launches them, hsmm::decode_tensor_viterbi_cuda
 * (src/hsmm.cu:604-720) and run_induction (src/hsmm.cu:731-791), launch for
 * launch:
 *   kernel_initialization   grid (N,N), min(next_pow2(D),1024) threads,
 *                           (2*bs + bs/32) doubles of shared memory
 *   per step t = 1..T-1     kernel_induction (N,N) x min(next_pow2(min(t,D)),1024)
 *                           with obs[t] by value and double-buffered em
 *                           windows, then kernel_reduce_i N x next_pow2(N)
 *   tail                    kernel_tail_adjustment (N,N), kernel_tail_reduce_i
 * followed by the copy of delta / psi_state / psi_dur (N x T, [j*T + t]) and
 * the host backtrace of src/hsmm.cu:139-170.  The binding's transposes of the
 * two duration tables (src/bindings.cpp:43-55) are done here too.
 *
 * Differences from the reference host code, none of which changes a value:
 * errors are returned (the reference exits, src/hsmm.cu:22-30); psi_state is
 * cleared once so the rows the reduction never writes (t < D, no update)
 * hold 0 as in the reference's host vector; the backtrace checks every
 * back-pointer before following it; the unused `d_emissions` buffer is not
 * allocated.  Inputs the reference does not check (T < D, observations out
 * of range, N above one block) are refused before anything is launched.
 */
#include <cuda.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>

#define TVR_OK 0
#define TVR_EINVAL -1
#define TVR_ESHORT -2
#define TVR_ERANGE -3
#define TVR_ENOMEM -4
#define TVR_ECUDA -5
#define TVR_ELOAD -6
#define TVR_EBACK -7

static char g_err[512];
const char* tvr_last_error(void) { return g_err; }

enum { K_INIT, K_IND, K_RED, K_TAIL, K_TRED, K_COUNT };
static const char* k_names[K_COUNT] = {"kernel_initialization", "kernel_induction", "kernel_reduce_i",
                                       "kernel_tail_adjustment", "kernel_tail_reduce_i"};
static CUmodule g_mod;
static CUfunction g_fn[K_COUNT];
static char g_loaded[1024];

#define CK(call)                                                                          \
    do {                                                                                  \
        CUresult r_ = (call);                                                             \
        if (r_ != CUDA_SUCCESS) {                                                         \
            const char* s_ = NULL;                                                        \
            cuGetErrorString(r_, &s_);                                                    \
            snprintf(g_err, sizeof g_err, "%s: %s", #call, s_ ? s_ : "?");                \
            rc = TVR_ECUDA;                                                               \
            goto done;                                                                    \
        }                                                                                 \
    } while (0)

static int next_pow2(int x) {
    if (x <= 1) return 1;
    unsigned u = (unsigned)(x - 1);
    u |= u >> 1; u |= u >> 2; u |= u >> 4; u |= u >> 8; u |= u >> 16;
    return (int)(u + 1);
}

static double now_ms(void) {
    struct timespec ts;
    clock_gettime(CLOCK_MONOTONIC, &ts);
    return ts.tv_sec * 1e3 + ts.tv_nsec * 1e-6;
}

/* A current context on device 0 (the reference uses device 0 implicitly):
 * the caller's, else the device's primary context. */
static int ensure_context(void) {
    int rc = TVR_OK;
    CUcontext c = NULL;
    CK(cuInit(0));
    CK(cuCtxGetCurrent(&c));
    if (!c) {
        CUdevice dev;
        CK(cuDeviceGet(&dev, 0));
        CK(cuDevicePrimaryCtxRetain(&c, dev));
        CK(cuCtxSetCurrent(c));
    }
done:
    return rc;
}

/* Loads the cubin and looks the five kernels up by the mangled names listed
 * in `names` ("<name> <mangled>" per line). */
static int load(const char* cubin, const char* names) {
    int rc = TVR_OK;
    if (g_mod && strcmp(g_loaded, cubin) == 0) return TVR_OK;
    char mangled[K_COUNT][256];
    memset(mangled, 0, sizeof mangled);
    FILE* f = fopen(names, "r");
    if (!f) {
        snprintf(g_err, sizeof g_err, "cannot open %s", names);
        return TVR_ELOAD;
    }
    char a[256], b[256];
    while (fscanf(f, "%255s %255s", a, b) == 2)
        for (int k = 0; k < K_COUNT; ++k)
            if (strcmp(a, k_names[k]) == 0) memcpy(mangled[k], b, sizeof b);
    fclose(f);
    for (int k = 0; k < K_COUNT; ++k)
        if (!mangled[k][0]) {
            snprintf(g_err, sizeof g_err, "%s not listed in %s", k_names[k], names);
            return TVR_ELOAD;
        }
    if ((rc = ensure_context()) != TVR_OK) return rc;
    CK(cuModuleLoad(&g_mod, cubin));
    for (int k = 0; k < K_COUNT; ++k) CK(cuModuleGetFunction(&g_fn[k], g_mod, mangled[k]));
    snprintf(g_loaded, sizeof g_loaded, "%s", cubin);
done:
    if (rc != TVR_OK) g_mod = NULL;
    return rc;
}

static int launch(CUfunction fn, unsigned gx, unsigned gy, unsigned bx, unsigned smem, void** args) {
    int rc = TVR_OK;
    CK(cuLaunchKernel(fn, gx, gy, 1, bx, 1, 1, smem, NULL, args, NULL));
done:
    return rc;
}

/*
 * Decodes one sequence with the reference CUDA kernels.  Arguments in the
 * reference binding's Python layouts (src/bindings.cpp:19-32): trans (N,N)
 * [to][from], emission (O,N), dur_lin (D,N) linear, start (N), dur (D,N),
 * obs (T) 0-based.  Outputs: path (T), *loglik = the best final score the
 * backtrace starts from, final (N, may be NULL) = delta[j][T-1] after the
 * tail, ms (may be NULL) = {whole call, kernels from the first launch to the
 * tail reduction (CUDA events)}.
 */
int tvr_decode(const char* cubin, const char* names, int N, int O, int D, int T, const double* trans,
               const double* emission, const double* dur_lin, const double* start, const double* dur,
               const int32_t* obs, int32_t* path, double* loglik, double* final, double* ms) {
    int rc = TVR_OK;
    if (N <= 0 || O <= 0 || D <= 0 || T <= 0 || !trans || !emission || !dur_lin || !start || !dur || !obs || !path) {
        snprintf(g_err, sizeof g_err, "bad argument");
        return TVR_EINVAL;
    }
    if (N > 1024) {
        snprintf(g_err, sizeof g_err, "N=%d: the reference's reduction takes next_pow2(N) <= 1024 threads", N);
        return TVR_EINVAL;
    }
    if (T < D) {
        snprintf(g_err, sizeof g_err, "T=%d < D=%d: the reference initialisation reads obs[0..D)", T, D);
        return TVR_ESHORT;
    }
    for (int t = 0; t < T; ++t)
        if (obs[t] < 0 || obs[t] >= O) {
            snprintf(g_err, sizeof g_err, "observation %d at t=%d outside [0,%d)", obs[t], t, O);
            return TVR_ERANGE;
        }
    if ((rc = load(cubin, names)) != TVR_OK) return rc;

    const double t_start = now_ms();
    const size_t NN = (size_t)N * N, ND = (size_t)N * D, NT = (size_t)N * T;
    double *dp = NULL, *dpl = NULL, *h_delta = NULL;
    int32_t *h_ps = NULL, *h_pd = NULL;
    CUdeviceptr d_tm = 0, d_em = 0, d_dpl = 0, d_sp = 0, d_dp = 0, d_obs = 0, d_delta = 0, d_AP = 0, d_APt = 0,
                d_vji = 0, d_dji = 0, d_ps = 0, d_pd = 0, d_w[2] = {0, 0};
    CUevent e0 = NULL, e1 = NULL;

    /* binding: duration tables (D,N) -> (N,D) */
    dp = (double*)malloc(sizeof(double) * ND);
    dpl = (double*)malloc(sizeof(double) * ND);
    h_delta = (double*)malloc(sizeof(double) * NT);
    h_ps = (int32_t*)malloc(sizeof(int32_t) * NT);
    h_pd = (int32_t*)malloc(sizeof(int32_t) * NT);
    if (!dp || !dpl || !h_delta || !h_ps || !h_pd) {
        snprintf(g_err, sizeof g_err, "host allocation failed");
        rc = TVR_ENOMEM;
        goto done;
    }
    for (int s = 0; s < N; ++s)
        for (int d = 0; d < D; ++d) {
            dp[(size_t)s * D + d] = dur[(size_t)d * N + s];
            dpl[(size_t)s * D + d] = dur_lin[(size_t)d * N + s];
        }

    /* hsmm_to_gpu (src/hsmm.cu:173-201) and the decode's own buffers (:624-646) */
    CK(cuMemAlloc(&d_tm, sizeof(double) * NN));
    CK(cuMemAlloc(&d_em, sizeof(double) * (size_t)O * N));
    CK(cuMemAlloc(&d_dpl, sizeof(double) * ND));
    CK(cuMemAlloc(&d_sp, sizeof(double) * N));
    CK(cuMemAlloc(&d_dp, sizeof(double) * ND));
    CK(cuMemAlloc(&d_obs, sizeof(int32_t) * T));
    CK(cuMemcpyHtoD(d_tm, trans, sizeof(double) * NN));
    CK(cuMemcpyHtoD(d_em, emission, sizeof(double) * (size_t)O * N));
    CK(cuMemcpyHtoD(d_dpl, dpl, sizeof(double) * ND));
    CK(cuMemcpyHtoD(d_sp, start, sizeof(double) * N));
    CK(cuMemcpyHtoD(d_dp, dp, sizeof(double) * ND));
    CK(cuMemcpyHtoD(d_obs, obs, sizeof(int32_t) * T));
    CK(cuMemAlloc(&d_delta, sizeof(double) * NT));
    CK(cuMemAlloc(&d_AP, sizeof(double) * ND * N));
    CK(cuMemAlloc(&d_APt, sizeof(double) * ND * N));
    CK(cuMemAlloc(&d_vji, sizeof(double) * NN));
    CK(cuMemAlloc(&d_dji, sizeof(int32_t) * NN));
    CK(cuMemAlloc(&d_ps, sizeof(int32_t) * NT));
    CK(cuMemAlloc(&d_pd, sizeof(int32_t) * NT));
    CK(cuMemAlloc(&d_w[0], sizeof(double) * ND));
    CK(cuMemAlloc(&d_w[1], sizeof(double) * ND));
    CK(cuMemsetD32(d_ps, 0, NT));
    CK(cuEventCreate(&e0, CU_EVENT_DEFAULT));
    CK(cuEventCreate(&e1, CU_EVENT_DEFAULT));
    CK(cuEventRecord(e0, NULL));

    /* phase 1: initialisation and the AP / AP_tail tables (src/hsmm.cu:648-658) */
    {
        const int bs = next_pow2(D) < 1024 ? next_pow2(D) : 1024;
        const unsigned sm = (unsigned)((2 * bs + bs / 32) * sizeof(double));
        void* a[] = {&d_sp, &d_dp, &d_dpl, &d_em, &d_obs, &d_delta, &d_pd, &d_tm, &d_AP, &d_APt, &N, &D, &T};
        if ((rc = launch(g_fn[K_INIT], N, N, bs, sm, a)) != TVR_OK) goto done;
    }
    /* phase 2: two launches per step (src/hsmm.cu:756-789) */
    {
        const int bsN = next_pow2(N);
        const unsigned sm_red = (unsigned)(bsN * (sizeof(double) + 2 * sizeof(int)));
        int cur = 0;
        for (int t = 1; t < T; ++t) {
            int tau = t < D ? t : D;
            const int nxt = 1 - cur;
            const int bs = next_pow2(tau) < 1024 ? next_pow2(tau) : 1024;
            const unsigned sm = bs > 32 ? (unsigned)((bs / 32) * (sizeof(double) + sizeof(int))) : 0u;
            int ot = obs[t];
            void* a[] = {&ot, &d_em, &d_delta, &d_AP, &d_w[cur], &d_w[nxt], &d_vji, &d_dji, &N, &D, &T, &tau, &t};
            if ((rc = launch(g_fn[K_IND], N, N, bs, sm, a)) != TVR_OK) goto done;
            void* b[] = {&d_vji, &d_dji, &d_delta, &d_ps, &d_pd, &N, &D, &T, &t};
            if ((rc = launch(g_fn[K_RED], N, 1, bsN, sm_red, b)) != TVR_OK) goto done;
            cur = nxt;
        }
        /* tail (src/hsmm.cu:668-695) */
        const int cur_final = (T - 1) % 2;
        const int tau_tail = (T - 1) < D ? (T - 1) : D;
        const int bs = next_pow2(tau_tail) < 1024 ? next_pow2(tau_tail) : 1024;
        const unsigned sm = bs > 32 ? (unsigned)(((bs + 31) / 32) * (sizeof(double) + sizeof(int))) : 0u;
        void* a[] = {&d_APt, &d_w[cur_final], &d_delta, &d_vji, &d_dji, &N, &D, &T};
        if ((rc = launch(g_fn[K_TAIL], N, N, bs, sm, a)) != TVR_OK) goto done;
        int tl = T - 1;
        void* b[] = {&d_vji, &d_dji, &d_delta, &d_ps, &d_pd, &N, &D, &T, &tl};
        if ((rc = launch(g_fn[K_TRED], N, 1, bsN, sm_red, b)) != TVR_OK) goto done;
    }
    CK(cuEventRecord(e1, NULL));
    CK(cuCtxSynchronize());
    CK(cuMemcpyDtoH(h_delta, d_delta, sizeof(double) * NT));
    CK(cuMemcpyDtoH(h_ps, d_ps, sizeof(int32_t) * NT));
    CK(cuMemcpyDtoH(h_pd, d_pd, sizeof(int32_t) * NT));

    /* backtracking_termination (src/hsmm.cu:139-170), with checks */
    {
        int t = T - 1, cur = 0;
        double best = h_delta[(size_t)0 * T + t];
        for (int n = 1; n < N; ++n)
            if (h_delta[(size_t)n * T + t] > best) { best = h_delta[(size_t)n * T + t]; cur = n; }
        if (final)
            for (int n = 0; n < N; ++n) final[n] = h_delta[(size_t)n * T + t];
        if (loglik) *loglik = best;
        while (t >= 0) {
            const int d = h_pd[(size_t)cur * T + t];
            const int prev = h_ps[(size_t)cur * T + t];
            if (d < 1 || d > t + 1 || prev < 0 || prev >= N) {
                snprintf(g_err, sizeof g_err, "back-pointer (d=%d, state=%d) at t=%d out of range", d, prev, t);
                rc = TVR_EBACK;
                goto done;
            }
            for (int k = t - d + 1; k <= t; ++k) path[k] = cur;
            t -= d;
            cur = prev;
        }
    }
    if (ms) {
        float kms = 0.0f;
        CK(cuEventElapsedTime(&kms, e0, e1));
        ms[1] = kms;
    }

done:
    if (e0) cuEventDestroy(e0);
    if (e1) cuEventDestroy(e1);
    CUdeviceptr bufs[] = {d_tm, d_em, d_dpl, d_sp, d_dp, d_obs, d_delta, d_AP, d_APt, d_vji, d_dji, d_ps, d_pd,
                          d_w[0], d_w[1]};
    for (size_t k = 0; k < sizeof bufs / sizeof bufs[0]; ++k)
        if (bufs[k]) cuMemFree(bufs[k]);
    free(dp);
    free(dpl);
    free(h_delta);
    free(h_ps);
    free(h_pd);
    if (ms && rc == TVR_OK) ms[0] = now_ms() - t_start;
    return rc;
}
