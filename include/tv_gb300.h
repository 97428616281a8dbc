/*
 * tv_gb300.h -- C ABI of the GB300 HSMM tensor-Viterbi decoder.
 *
 * Plain pointers and sizes only.  Every array is row-major and float64 unless
 * stated otherwise, in the Python-facing layouts of the reference binding
 * (src/bindings.cpp:19-32):
 *   trans_mat             (N, N) log space, indexed [to j][from i]
 *   emission_probs        (O, N) log space
 *   duration_probs_linear (D, N) linear space (accepted, not read: the
 *                         decoder follows the reference C++ backend, whose
 *                         tail uses the log-space survival function)
 *   start_probs           (N,)   log space
 *   duration_probs        (D, N) log space
 *   obs_seq               (T,)   0-based symbols, int32
 * The decoded path is int32 (T,).  The path log-likelihood is the
 * tail-adjusted score of the best final state, the value the reference's
 * backtrace starts from (src/hsmm.cu:147-155).
 *
 * Errors are returned as TV_* status codes; the library never exits the
 * process.  tv_last_error() gives a message for the calling thread.
 */
#ifndef TV_GB300_H
#define TV_GB300_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

enum tv_status {
    TV_OK = 0,
    TV_EINVAL = -1,     /* bad argument: size, null pointer, shape */
    TV_ESHORT = -2,     /* T < D: the reference initialisation reads obs[0..D) */
    TV_ERANGE = -3,     /* an observation outside [0, O) */
    TV_ENONFINITE = -4, /* NaN or +-inf in a model table */
    TV_ETOOBIG = -5,    /* N or D above 65536, or T above 2^31-1 */
    TV_ENOMEM = -6,     /* device or host allocation failed */
    TV_ECUDA = -7,      /* CUDA runtime error (see tv_last_error) */
    TV_EINTERNAL = -8,  /* device-side consistency check failed */
    TV_ENODEV = -9,     /* no CUDA device */
    TV_ETIMEOUT = -10,  /* a bounded device-side wait gave up (no progress) */
    TV_ENONPOS = -11    /* forward-backward: a normaliser or forward variable
                           not positive (hsmmlearn's err = 1) */
};

/* Message for the last non-OK status returned on this thread. */
const char* tv_last_error(void);

/*
 * One-shot decode with host buffers: the drop-in for the reference's
 * hsmm::decode_tensor_viterbi_cuda (src/hsmm.hpp:48-56, src/hsmm.cu:604-720)
 * as bound by src/bindings.cpp:104-114 and called from
 * tensor_viterbi/viterbi/native.py:67-81.  Same arguments; the caller owns
 * path_out (T int32).  loglik_out may be NULL.  Synchronous; device 0.
 */
int tv_decode_tensor_viterbi_cuda(int n_states, int n_symbols, int max_dur, int64_t T,
                                  const double* trans_mat, const double* emission_probs,
                                  const double* duration_probs_linear, const double* start_probs,
                                  const double* duration_probs, const int32_t* obs_seq,
                                  int32_t* path_out, double* loglik_out);

/*
 * Device-resident model: the tables the reference uploads per call in
 * hsmm_to_gpu (src/hsmm.cu:173-201), uploaded once and reused.  Host
 * pointers in the layouts above.  tv_model_destroy frees it.
 */
typedef struct tv_model_s* tv_model;
int tv_model_create(int n_states, int n_symbols, int max_dur,
                    const double* trans_mat, const double* emission_probs,
                    const double* duration_probs_linear, const double* start_probs,
                    const double* duration_probs, tv_model* out);
int tv_model_destroy(tv_model m);

/* Decode one sequence with host buffers through a model (synchronous).
 * Replaces the per-call body of src/hsmm.cu:604-720 after the upload. */
int tv_decode(tv_model m, const int32_t* obs_seq, int64_t T,
              int32_t* path_out, double* loglik_out);

/* Decode one sequence whose observations are already in device memory.
 * obs_dev (T int32), path_dev (T int32) and loglik_dev (1 double, may be
 * NULL) are device pointers; the call is asynchronous on `stream`
 * (a cudaStream_t, NULL = legacy default stream).  Scratch memory is owned
 * by the model and reused; calls on one model must not overlap. */
int tv_decode_device(tv_model m, const int32_t* obs_dev, int64_t T,
                     int32_t* path_dev, double* loglik_dev, void* stream);

/* Batched decode: n_seq independent sequences that share the model, in one
 * persistent launch.  No reference counterpart (the reference decodes one
 * sequence per call); each result equals the single-sequence decode.
 * obs_cat holds the sequences back to back, offsets[k]..offsets[k+1]
 * (n_seq+1 int64 entries) delimit sequence k, and path_cat has the same
 * shape.  Host buffers, synchronous.  loglik_out (n_seq) may be NULL. */
int tv_decode_batch(tv_model m, int n_seq, const int64_t* offsets,
                    const int32_t* obs_cat, int32_t* path_cat, double* loglik_out);

/* Device-pointer form of tv_decode_batch (asynchronous on `stream`);
 * offsets stays a host array, obs_cat/path_cat/loglik_dev are device
 * pointers. */
int tv_decode_batch_device(tv_model m, int n_seq, const int64_t* offsets,
                           const int32_t* obs_cat_dev, int32_t* path_cat_dev,
                           double* loglik_dev, void* stream);

/* Number of kernel launches the most recent decode on this model issued
 * (diagnostics for benchmark reporting). */
int64_t tv_model_last_launches(tv_model m);

/* Kernel selection for single-sequence decodes (no reference counterpart):
 * TV_PATH_AUTO picks the one-CTA kernel when the D-deep window fits one
 * CTA's shared memory and the whole-GPU grid kernel otherwise;
 * TV_PATH_CTA / TV_PATH_GRID force one of them.  The grid kernel keeps the
 * window in its workers' shared memory, or in global memory (L2) when it
 * does not fit there; TV_PATH_GRID_L2 forces the latter.  grid_ctas > 0
 * caps the grid kernel's CTA count (0 = one per SM).  All give identical
 * results. */
enum tv_path { TV_PATH_AUTO = 0, TV_PATH_CTA = 1, TV_PATH_GRID = 2, TV_PATH_GRID_L2 = 3 };
int tv_model_set_path(tv_model m, int path, int grid_ctas);

/* Which kernel the most recent single-sequence decode used (TV_PATH_CTA or
 * TV_PATH_GRID). */
int tv_model_last_path(tv_model m);

/* Threads per CTA of the most recent batched decode on this model, 0 before
 * any (no reference counterpart).  The batched decodes (tv_decode_batch,
 * tv_decode_batch_device) take the CTA shape from an autotuner: the first
 * batch of a (N, D) shape with at least two waves of CTAs runs every
 * candidate shape (128, 256, 384, 512 threads) for one wave of its own grid
 * on sequences of 2 D to 8 D steps cut from the batch's observations,
 * waiting for those runs, and the shape with the most steps per second is
 * kept for the process.  The trial runs write the batch's output buffers,
 * which the real decode then overwrites.  Setting the environment variable
 * TV_AUTOTUNE=0 keeps the default shape (256).  Results never depend on the
 * shape. */
int tv_model_batch_threads(tv_model m);
/* The number of CTAs of the last batched launch (the SM count times the CTAs
 * that share an SM, at most one per sequence); 0 before any. */
int tv_model_batch_grid(tv_model m);

/* Failure injection for tests (no reference counterpart; the reference's
 * answer to any device failure is exit(EXIT_FAILURE), src/hsmm.cu:22-30).
 * The next grid-kernel decode on this model loses one message: the worker
 * partial of `step` for worker segment `segment` is never sent.  The head's
 * bounded wait for it (or a worker's wait for the head, whichever gives up
 * first) runs out after about a second of SM clocks; every CTA then leaves
 * at the same step and the decode returns TV_ETIMEOUT, naming the wait.
 * Applies to one decode; later decodes are unaffected. */
int tv_model_drop_partial(tv_model m, int64_t step, int segment);

/* The whole-GPU grid kernel's plan for a shape, computed on the host alone
 * (diagnostics and tests; no reference counterpart; no GPU needed).  For N
 * states, D durations, G CTAs (the head and G-1 workers) and a per-CTA
 * shared-memory limit, fills out[0..9] = {plan exists (1/0), threads per
 * CTA, dynamic shared bytes per CTA, window in global memory (1/0), matvec
 * split over two warps per 32 states (1/0), worker segments S, most
 * segments of one worker, head threads with a role, fixed-point duration
 * rows in shared memory with the window in global memory (1/0), workers
 * that own cells}. */
int tv_grid_plan_info(int N, int D, int G, int smem_optin, int force_l2, int64_t* out);

/* Per-step latency floor of the grid decoder (diagnostics for benchmark
 * reporting; no reference counterpart).  Runs, alone on one SM, the part of
 * a step that only the head's critical lanes can do -- the packed N x N
 * matvec with the grid plan's layout for (n_states, max_dur), the exact d = 0
 * score, its fixed-point re-pack and the step barrier -- for `steps` steps,
 * then bounces a tagged word between two SMs 2000 times.  out[0..6] = {clocks
 * per step, microseconds per step (CUDA events), clocks per cross-SM round
 * trip, microseconds per round trip, matvec split (1/0), SM ids of the two
 * round-trip CTAs}.  Synchronous; allocates and frees its own buffers. */
int tv_step_floor(int n_states, int max_dur, int64_t steps, double* out);

/* One SM's FP64 unit (diagnostics for benchmark reporting; no reference
 * counterpart): the bound of tv_fb, whose sequence runs on one SM.
 * out[0..3] = {FP64 warp instructions per clock with 8 warps of 8
 * independent fused multiply-add chains, that SM's FP64 FLOP/s (an FMA is two,
 * CUDA events), the SM clock over the run in MHz, clocks per dependent FP64
 * instruction of one warp}.  Synchronous. */
int tv_fp64_peak(double* out);

/* Device time in milliseconds of the calling thread's last tv_fb kernel
 * (CUDA events around its launch; copies excluded); 0 before any call. */
double tv_fb_last_kernel_ms(void);

/* Kernel timing for benchmark reporting (no reference counterpart).  When
 * enabled, CUDA events on the decode's own stream bracket its main kernel;
 * tv_model_kernel_ms waits for that kernel and returns its time in ms for
 * the most recent decode, or a negative value when none was recorded. */
int tv_model_set_timing(tv_model m, int enable);
double tv_model_kernel_ms(tv_model m);

/*
 * Decode one sequence without allocating device memory (no counterpart in the
 * reference).  For callers that must not call cudaMalloc at decode time:
 * code running inside a CUDA graph capture or a stream callback, real-time
 * or latency-critical loops where an allocation can stall on the driver, and
 * processes whose device memory is fully reserved up front by a pool.  The
 * model (tv_model_create) is the only allocation, made once at set-up.
 *
 * Scratch (the fixed-point tables for this decode, the back-pointers and a
 * few control words) comes from one fixed array compiled into the library,
 * TV_STATIC_SCRATCH_BYTES large, that every GPU using the library holds until
 * the process exits.  Limits: the scratch a decode needs,
 *     r(8*O*N) + r(8*N*N) + r(8*N*D) + 256 + 4*T*N bytes,
 * with r(x) = x rounded up to a multiple of 256 (three tables, the control
 * words, the back-pointers), must fit in it, and the D-deep window must fit
 * one CTA's shared memory (34*N*D + 8*N*N bytes <= 227 KB); larger problems
 * return TV_ETOOBIG before anything is launched.
 *
 * The first call on a device looks the array up (cudaGetSymbolAddress) and
 * sets the kernel's shared-memory attribute with that device current; make
 * that first call before any stream capture.  All calls share the one array
 * and leave their data in it: calls that overlap on the GPU (other streams,
 * other threads, other models) race; serialise them.  obs_dev, path_dev
 * (T int32), loglik_dev (1 double) and status_dev (1 int, 0 on success, or a
 * TV_* code such as TV_ERANGE for an observation outside [0, O)) are device
 * pointers; loglik_dev and status_dev may be NULL.  Asynchronous on `stream`.
 */
#define TV_STATIC_SCRATCH_BYTES (32u << 20)
int tv_decode_device_static(tv_model m, const int32_t* obs_dev, int64_t T,
                            int32_t* path_dev, double* loglik_dev, int* status_dev,
                            void* stream);

/* ---- HSMM training: the forward-backward E step ----
 *
 * tv_fb replaces hsmmlearn's FBImpl (hsmmlearn/hsmmlearn/_hsmm/src/FBImpl.cpp)
 * as called through its wrapper _fb_impl (hsmmlearn/hsmmlearn/base.pyx:50-)
 * by HSMMModel.fit (hsmmlearn/hsmmlearn/hsmm.py:181-305) once per EM
 * iteration.  Same arguments and layouts, host buffers, synchronous:
 *   censoring  0 none, 1 right censoring (fit's default); 2 (left and right)
 *              is not supported and returns TV_EINVAL
 *   d (J, M)   duration pmf rows, entry u-1 = P(duration u)
 *   p (J, J)   transition matrix [from][to]; pi (J); pdf (J, tau) likelihoods
 *   outputs    F, L, G, L1, Norm (J, tau), N (tau), eta (J, M); G[:, 0] and
 *              L1[:, tau-1] are not written (left as passed in)
 * Returns TV_OK, or TV_ENONPOS where the reference reports err = 1.  Values
 * agree with the reference to rounding (some products and sums associate
 * differently), not bit for bit. */
int tv_fb(int censoring, int64_t tau, int J, int M, const double* d, const double* p, const double* pi,
          const double* pdf, double* F, double* L, double* G, double* L1, double* N, double* Norm,
          double* eta);

/* ---- Gaussian emissions (no reference counterpart: the reference takes a
 * discrete emission table only; a per-timestep table with obs = 0..T-1 is
 * the same decode) ----
 *
 * tv_gaussian_loglik: the emission front-end on the device.  table_dev
 * (T x N, row t = observation t) receives log N(x_t; mean_j, sd_j) =
 * ((-0.5 z) z - log sd_j) - log(2 pi)/2 with z = (x_t - mean_j) / sd_j, every
 * operation rounded once in FP64 and log sd_j, log(2 pi) taken on the host
 * with the C library's log, so the table equals that expression evaluated on
 * the host.  x_dev is a device array of T doubles; mean and sd are host
 * arrays of N.  Asynchronous on `stream`.
 *
 * tv_model_create_gaussian: a model whose emission table is built that way
 * from host observations x (T doubles); decode it with obs = 0..T-1. */
int tv_gaussian_loglik(const double* x_dev, int64_t T, int n_states, const double* mean,
                       const double* sd, double* table_dev, void* stream);
int tv_model_create_gaussian(int n_states, int max_dur, int64_t T, const double* trans_mat,
                             const double* duration_probs_linear, const double* start_probs,
                             const double* duration_probs, const double* x, const double* mean,
                             const double* sd, tv_model* out);

/* ---- Decode server (no reference counterpart): continuous batching of
 * independent requests, each with its own model. ----
 *
 * A scheduler thread admits submitted requests in arrival order while the
 * device-memory budget allows (budget_bytes <= 0: 80% of the free memory)
 * and one of max_inflight streams is free (<= 0: 64).  Each admitted request
 * runs on its own stream with its own model and buffers, allocated in stream
 * order, so requests overlap on the GPU and each result is the one a decode
 * alone gives.  Submission copies the inputs and returns a ticket >= 0 (or a
 * negative status).  tv_server_poll returns 1 and writes the path (T int32),
 * the log-likelihood and latency_ms_out[0..1] = {submission to completion,
 * submission to admission} when the request is done (the ticket is then
 * released), 0 while it is pending, or the request's negative status;
 * tv_server_wait blocks until done.  tv_server_stats writes 8 counters:
 * admitted, completed, failed, running, pending, bytes in use, peak bytes in
 * use, budget.  tv_server_destroy finishes the requests in flight. */
typedef struct tv_server_s* tv_server;
tv_server tv_server_create(int64_t budget_bytes, int max_inflight);
int tv_server_destroy(tv_server s);
int64_t tv_server_submit(tv_server s, int n_states, int n_symbols, int max_dur, int64_t T,
                         const double* trans_mat, const double* emission_probs,
                         const double* duration_probs_linear, const double* start_probs,
                         const double* duration_probs, const int32_t* obs_seq);
int64_t tv_server_submit_gaussian(tv_server s, int n_states, int max_dur, int64_t T,
                                  const double* trans_mat, const double* duration_probs_linear,
                                  const double* start_probs, const double* duration_probs,
                                  const double* x, const double* mean, const double* sd);
int tv_server_poll(tv_server s, int64_t ticket, int32_t* path_out, double* loglik_out,
                   double* latency_ms_out);
int tv_server_wait(tv_server s, int64_t ticket, int32_t* path_out, double* loglik_out,
                   double* latency_ms_out);
int tv_server_stats(tv_server s, int64_t* out);

#ifdef __cplusplus
}
#endif
#endif
