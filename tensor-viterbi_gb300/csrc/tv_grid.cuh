// tv_grid.cuh -- one sequence decoded by the whole GPU: a persistent,
// co-resident grid of one head CTA and G-1 worker CTAs.
//
// The D-deep window of the recurrence (N*D cells) is spread over the workers
// and stays in their shared memory for the whole decode; nothing of it goes
// back to HBM per step.  Cell (j, r) is ring slot r of state j: it holds the
// predecessor end s with s % D == r, so at step t its duration index is
// d = (t-1-s) and it turns over every D steps without moving.
//
// Per step t:
//   head    the serial critical path, all in its own shared memory: the N x N
//           max-plus matvec for the newest slot s = t-1 (sent to the workers),
//           the candidates d < L, the merge with the workers' exact partial
//           winners, the initialisation rule for t < D, the exact delta[t]
//           and the back-pointers.
//   workers for their cells: the fixed-point scan over d >= L, the certified
//           exact local winner (sent to the head), and, overlapped with it,
//           the exact window folds of step t+1 (double-buffered).  A worker
//           needs slot t-1-L to run step t, so it runs up to L steps ahead of
//           the head and the cross-SM latency is overlapped, not paid per
//           step.
// Every cross-CTA value travels as tagged 64-bit words (tv_sync.cuh): a reader
// that sees the expected tag holds the value, so no fence or flag round trip
// sits on any per-step path.
// After step T-1 the tail (survival in place of the duration pmf) is one more
// round of the same protocol with an exhaustive exact scan; the head then
// backtraces.
//
// While t <= D the reference rebuilds the window sums newest-first
// (src/hsmm.cu:311-322); a worker then takes the exact value of its winner
// from a checkpoint table g_t(k*K) built before the launch plus at most K-1
// additions.
#pragma once
#include <climits>

#include "tv_cta.cuh"
#include "tv_device.cuh"
#include "tv_sync.cuh"

namespace tv {

constexpr int GRID_THREADS = 640;    // largest block (96 registers a thread)
constexpr int WORKER_THREADS = 256;     // a worker CTA's scan threads: 8 warps (window in shared memory)
constexpr int WORKER_THREADS_GW = 512;  // 16 warps when the window is in global memory (more loads in flight)
constexpr int WORKER_SERVICE = 64;      // + a certify warp and an intake warp; the rest of the CTA exits
constexpr int GRID_L = 8;            // head candidates d < L (a power of two)
constexpr int CK_STRIDE = 32;      // checkpoint stride of the early window sums
constexpr int PART_RING = 32;      // steps of worker partials in flight
constexpr int SLOT_RING = 64;      // slot messages kept
constexpr int SLOT_WORDS = 5;      // ctil (2), dsel (2), itil (1)
constexpr int GRID_MAX_N = 128;    // packed coarse scores keep the state index in 7 bits
constexpr int COARSE_F = 14;       // fraction bits of the packed coarse matvec scores
constexpr int COARSE_CLAMP = (1 << 23) - 1;
constexpr int EMPTY_D = 0xffff;
constexpr int TV_ETIMEOUT_DEV = -10;

struct GridParams {
  int G, L, S, Rd, M;
  long long chunk;  // largest worker range, in cells
  int max_seg;
  unsigned long long w_qd, w_dur, w_tr, w_ctil, w_dsel, w_acc, w_accs, w_itil, w_red, w_emw, w_bytes;
  int w_global;                  // the window lives in global memory (L2), not in shared memory
  unsigned long long w_gstride;  // bytes of one worker's window in global memory
  int w_qd_smem;                 // window in global memory, fixed-point duration rows in shared memory
  // head shared-memory offsets
  unsigned long long h_xch, h_qcp, h_qtr, h_trh, h_dqcp, h_dq, h_ptil, h_base, h_dstar, h_ctil, h_itil, h_hwr, h_qd, h_dur,
      h_prek, h_pred, h_prei, h_prew, h_preq, h_pwq, h_pwk, h_pwd, h_pwi, h_psirec, h_tail, h_bytes;
  int trans_smem;     // the exact transition matrix is kept in the head's shared memory
  int qtr_smem;       // so is its fixed-point copy (else computed from the exact one)
  int st_threads;     // state helper threads per group (two groups): N rounded up to 32
  int in_threads;     // intake threads: max(ceil(S/2), N) rounded up to 32
  int block;          // threads per CTA: the head's roles (at least a worker's scan and service threads)
  int qf;             // fraction bits of the fixed-point scores
  int Np;             // N rounded up to 16 (packed coarse matvec rows)
  int cs_threads;     // critical threads: one lane per state, N rounded up to 32
  int cs_split;       // 1: a second warp per 32 states scans the upper half of i in the matvec
  int coarse_shift;   // fine-to-coarse right shift (f - COARSE_F)
  int coarse_margin;  // certified coarse i-margin, coarse units
  long long timeout;
  long long copy_timeout;  // the head's wait for its own window-sum copies: fixed, so a copy is always drained
  // Test-only fault injection (tv_model_drop_partial): the worker partial of
  // step drop_tag for segment drop_seg is not sent, as if the message were
  // lost; 0 = none (tags start at 1).
  unsigned drop_tag;
  int drop_seg;
};

struct GridBufs {
  const int32_t* obs;
  long long T;
  uint32_t* psi;                // (T, N)
  int32_t* path;                // (T)
  double* loglik;               // (1) or null
  unsigned long long* slot_msg; // [SLOT_RING][N][5] tagged slot records
  unsigned long long* part;     // [PART_RING][S][3] tagged partial winners
  unsigned long long* dstar;    // [Rd][N][2] tagged exact delta ring
  const double* dinit;          // [D][N] initialisation scores
  const double* ck;             // [D][M][N] checkpoints of the early window sums
  const double* hwin;           // [T][L][N] window sums E_t[d], d < L
  const long long* wrange;      // [G-1][2] worker cell ranges
  unsigned char* wglob;         // [G-1][w_gstride] worker windows when they do not fit shared memory
  const int* seg_first;         // [N]
  const int* seg_count;         // [N]
  const int* seg_base;          // [G-1]
  int* abort_flag;
  int* status;
  int* site;                    // which wait gave up (diagnostics)
};

// g_t(d) = em_t + em_{t-1} + ... + em_{t-d}, folded newest-first like the
// reference's rebuild for t <= D, from the checkpoint at K*floor(d/K).
__device__ __forceinline__ double early_window(const ModelView& m, const double* ck, int M, const int32_t* obs,
                                               long long t, int d, int j) {
  const int q = d / CK_STRIDE;
  double g = ck[((size_t)(t - 1) * M + q) * m.N + j];
  for (int k = q * CK_STRIDE + 1; k <= d; ++k) g = g + m.em[(size_t)obs[t - k] * m.N + j];
  return g;
}

// Window sum E_t[d] (d < min(t, D)) as the reference holds it at step t, from
// an accessor em(s) of the emission values: newest-first while t <= D
// (src/hsmm.cu:311-322); after that the rolling fold E_t[d] = E_{t-1}[d-1] +
// em_t (src/hsmm.cu:298-310) unrolled back to where it began: 0 + em_{t-d}
// then oldest-first, or, when it reaches back to step D, the newest-first sum
// of step D then oldest-first.
template <class F>
__device__ __forceinline__ double window_sum(F em, int D, long long t, int d) {
  double g;
  if (t <= D) {
    g = em(t);
    for (int k = 1; k <= d; ++k) g = g + em(t - k);
    return g;
  }
  long long s0 = t - d;
  if (s0 > D) {
    g = 0.0 + em(s0);
  } else {
    const int dd = d - (int)(t - D);
    g = em(D);
    for (int k = 1; k <= dd; ++k) g = g + em(D - k);
    s0 = D;
  }
  for (long long s = s0 + 1; s <= t; ++s) g = g + em(s);
  return g;
}

// The head's window sums E_t[d] for d < L at every step, [T][L][N] (zero where
// d >= min(t, D)): read a few steps ahead by the head instead of folded on
// its critical path.
__global__ void grid_prep_hwin(ModelView m, const int32_t* obs, long long T, double* hwin, const int* abort_flag) {
  const long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (idx >= T * m.N || *abort_flag) return;
  const long long t = idx / m.N;
  const int j = (int)(idx % m.N);
  const int tau = (int)(t < m.D ? t : m.D);
  auto em = [&](long long s) { return m.em[(size_t)obs[s] * m.N + j]; };
  double* out = hwin + (size_t)t * GRID_L * m.N + j;
  for (int d = 0; d < GRID_L; ++d) out[(size_t)d * m.N] = d < tau ? window_sum(em, m.D, t, d) : 0.0;
}

// Observations may come straight from device memory: a value outside [0, O)
// raises the abort word (status TV_ERANGE) and every later kernel of the
// decode returns before reading the tables with it.
__global__ void grid_check_obs(const int32_t* obs, long long T, int O, int* abort_flag, int* status) {
  for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < T; t += (long long)gridDim.x * blockDim.x)
    if ((unsigned)obs[t] >= (unsigned)O) {
      atomicExch(abort_flag, 1);
      atomicCAS(status, 0, -3);
    }
}

// Initialisation scores delta[t][j] = (dur[j][t] + start[j]) + E0[t][j] for
// t < D, E0 the oldest-first running emission sum (src/hsmm.cu:274-290).
__global__ void grid_prep_init(ModelView m, const int32_t* obs, double* dinit, const int* abort_flag) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= m.N || *abort_flag) return;
  double e = 0.0;
  const double sj = m.start[j];
  for (int d = 0; d < m.D; ++d) {
    e = e + m.em[(size_t)obs[d] * m.N + j];
    dinit[(size_t)d * m.N + j] = (m.durT[(size_t)j * m.D + d] + sj) + e;
  }
}

// Checkpoints g_t(k*K) of the newest-first window sums for 1 <= t <= tmax.
__global__ void grid_prep_ck(ModelView m, const int32_t* obs, double* ck, int M, int tmax, const int* abort_flag) {
  const long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (idx >= (long long)tmax * m.N || *abort_flag) return;
  const int t = (int)(idx / m.N) + 1;
  const int j = (int)(idx % m.N);
  double* row = ck + (size_t)(t - 1) * M * m.N + j;
  double g = m.em[(size_t)obs[t] * m.N + j];
  row[0] = g;
  for (int d = 1; d < t; ++d) {
    g = g + m.em[(size_t)obs[t - d] * m.N + j];
    if (d % CK_STRIDE == 0) row[(size_t)(d / CK_STRIDE) * m.N] = g;
  }
}

// Wait sites reported with a timeout.
enum { SITE_HEAD_PARTIAL = 1, SITE_WORKER_SLOT = 2, SITE_WORKER_RESCORE = 3, SITE_WORKER_TAIL = 4,
       SITE_HEAD_TAIL = 5, SITE_HEAD_COPY = 6 };

__device__ __forceinline__ void grid_fail(const GridBufs& B, int code, int site) {
  if (atomicCAS(B.status, 0, code) == 0) *B.site = site;
  atomicExch(B.abort_flag, 1);
}

// A slot message (score, selected delta, argmax word) in one round trip:
// the five words are loaded together and polled until each carries `tag`.
__device__ __forceinline__ bool slot_load(const unsigned long long* src, unsigned tag, unsigned long long& cbits,
                                          unsigned long long& dbits, unsigned& ibits, const int* abort_flag,
                                          long long limit) {
  unsigned long long w[SLOT_WORDS];
#pragma unroll
  for (int k = 0; k < SLOT_WORDS; ++k) w[k] = ld_relaxed_u64(src + k);
  auto ready = [&]() {
    bool ok = true;
#pragma unroll
    for (int k = 0; k < SLOT_WORDS; ++k) ok = ok && (unsigned)(w[k] >> 32) == tag;
    return ok;
  };
  if (!ready()) {
    const long long t0 = clock64();
    for (;;) {
      __nanosleep(20);
#pragma unroll
      for (int k = 0; k < SLOT_WORDS; ++k) w[k] = ld_relaxed_u64(src + k);
      if (ready()) break;
      if (ld_relaxed_i32(abort_flag)) return false;
      if (clock64() - t0 > limit) return false;
    }
  }
  cbits = (w[0] & 0xffffffffull) | ((w[1] & 0xffffffffull) << 32);
  dbits = (w[2] & 0xffffffffull) | ((w[3] & 0xffffffffull) << 32);
  ibits = (unsigned)(w[4] & 0xffffffffull);
  return true;
}

// Exact delta[s][i] from the tagged ring (tag s+1), as an order key.
__device__ __forceinline__ bool load_dstar(const GridBufs& B, const GridParams& P, int N, long long s, int i,
                                           double& v) {
  unsigned long long bits;
  if (!tagged64_load(B.dstar + ((size_t)(s % P.Rd) * N + i) * 2, (unsigned)(s + 1), bits, B.abort_flag, P.timeout))
    return false;
  v = __longlong_as_double((long long)bits);
  return true;
}

// Named barriers of a worker CTA: 1 for its scan threads, 2 for the scan
// threads with the service warps (the rest of the CTA has exited).  The
// non-aligned barrier counts threads, so lanes of a warp may arrive apart
// (after a lane-0 wait, say); the aligned bar.sync would need the warp
// converged, which the compiler does not ensure before inline assembly.
template <int WT>
__device__ __forceinline__ void worker_sync() {
  asm volatile("barrier.sync 1, %0;" ::"r"(WT) : "memory");
}
template <int WT>
__device__ __forceinline__ void worker_sync_all() {
  asm volatile("barrier.sync 2, %0;" ::"r"(WT + WORKER_SERVICE) : "memory");
}

// Block-wide reduction of an ExactBest over the worker threads; every worker
// thread receives the result.
template <int WT>
__device__ __forceinline__ ExactBest worker_reduce_exact(ExactBest eb, ExactBest* scratch) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  eb.warp_reduce();
  worker_sync<WT>();
  if (lane == 0) scratch[warp] = eb;
  worker_sync<WT>();
  ExactBest r;
  r.init();
  if (lane < WT / 32) r = scratch[lane];
  r.warp_reduce();
  return r;
}

__device__ __forceinline__ void send_partial(const GridBufs& B, const GridParams& P, unsigned tag, unsigned ring,
                                             int seg, const ExactBest& eb) {
  if (tag == P.drop_tag && seg == P.drop_seg) return;  // test-only: a lost message
  TaggedMsg msg;
  const bool empty = eb.d == IDX_NONE;
  // the winner's order key and fixed-point value, and (d, i)
  msg_pack(msg, tag, eb.k, empty ? 0 : fixed_from_double(eb.value(), P.qf),
           empty ? ((unsigned)EMPTY_D << 16) : (((unsigned)eb.d << 16) | (unsigned)eb.i));
  msg_store(B.part + ((size_t)ring * P.S + seg) * MSG_WORDS, msg);
}

// ---------------------------------------------------------------------------
// Worker CTA: WORKER_THREADS scan threads (WORKER_THREADS_GW with the window
// in global memory) and two service warps, run as a software pipeline.
// Step t:
//   scan threads   phase 1: the fixed-point scan of the worker's cells over
//                  d in [L, tau) (best and runner-up per segment), fused with
//                  the exact window folds of step t+1;
//   certify warp   (during phase 1 of step t+1) the certified exact winner of
//                  each segment at step t, sent to the head;
//   intake warp    (during phase 1 of step t+1) the slot that enters the scan
//                  at step t+2 (s' = t+1-L, d = L then), from the head.
// So the window sums are kept in three buffers (E_t, E_{t+1}, E_{t+2}) and the
// per-warp scan results in two (by step parity).
// ---------------------------------------------------------------------------
// GW: the worker's window (slot scores, selected deltas, window sums, argmax
// words) lives in a private global-memory buffer, served by L1/L2, and the
// exact duration and transition rows are read from the model's tables; used
// when N*D is too large for the workers' shared memory.  The fixed-point
// duration rows, read every step by the scan, stay in shared memory when they
// fit there (P.w_qd_smem).
template <bool GW>
__device__ void grid_worker(const ModelView& m, const GridParams& P, const GridBufs& B, unsigned char* sm) {
  constexpr int L = GRID_L;
  constexpr int WT = GW ? WORKER_THREADS_GW : WORKER_THREADS;
  constexpr int NW = WT / 32;
  static_assert(NW <= 32 && (32 % NW) == 0, "segment groups of the certify warp");
  const int N = m.N, D = m.D;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int w = blockIdx.x - 1;
  const long long c_lo = B.wrange[2 * w], c_hi = B.wrange[2 * w + 1];
  if (c_lo >= c_hi) return;  // idle worker: owns no cells, sends nothing
  const int ja = (int)(c_lo / D), jb = (int)((c_hi - 1) / D);
  const int nseg = jb - ja + 1;
  const int off0 = (int)(c_lo - (long long)ja * D);  // ring slot of the first cell
  const int seg0 = B.seg_base[w];
  const long long T = B.T;
  unsigned char* wb = GW ? B.wglob + (size_t)w * P.w_gstride : sm;
  long long* qd_s = (long long*)(sm + P.w_qd);        // [nseg][D]
  double* dur_s = (double*)(sm + P.w_dur);            // [nseg][D]
  double* tr_s = (double*)(sm + P.w_tr);              // [nseg][N]
  const bool qd_in_smem = !GW || P.w_qd_smem;
  const long long* qd = qd_in_smem ? qd_s : m.qdurT + (size_t)ja * D;
  const double* dur = GW ? m.durT + (size_t)ja * D : dur_s;
  const double* tr = GW ? m.trans + (size_t)ja * N : tr_s;
  long long* ctil = (long long*)(wb + P.w_ctil);      // [ncell]
  double* dsel = (double*)(wb + P.w_dsel);            // [ncell]
  double* accb = (double*)(wb + P.w_acc);             // [3][ncell] E_t in buffer t % 3
  const size_t accs = P.w_accs / sizeof(double);
  unsigned short* itil = (unsigned short*)(wb + P.w_itil);
  Top2* red = (Top2*)(sm + P.w_red);                  // [2][nseg][NW] by step parity
  ExactBest* ered = (ExactBest*)(sm + P.w_red);
  double* emw = (double*)(sm + P.w_emw);              // [2][max_seg] emission of the fold's step
  // Failure flags by step parity: set by the service warps of step t, read
  // by every thread after the barrier that ends their work, so that all
  // leave at the same step.
  __shared__ int s_bad[2];
  const bool is_scan = tid < WT;

  // Fixed-point durations below L are masked in the worker's copy: with every
  // fixed-point score below 2^61 in magnitude, a masked cell scores below
  // QNEG and never enters a scan's best or runner-up, so the scan needs no
  // range test once tau = D.
  constexpr long long QMASK = -(3LL << 61);
  if (is_scan && qd_in_smem)
    for (long long k = tid; k < (long long)nseg * D; k += WT) qd_s[k] = (k % D) < L ? QMASK : m.qdurT[(size_t)ja * D + k];
  if (is_scan && !GW) {
    for (long long k = tid; k < (long long)nseg * D; k += WT) dur_s[k] = m.durT[(size_t)ja * D + k];
    for (int k = tid; k < nseg * N; k += WT) tr_s[k] = m.trans[(size_t)ja * N + k];
  }
  // Slot scores start at 0: a cell whose first slot has not arrived yet is
  // read (masked) by the unpredicated scan, and must hold a bounded value.
  if (is_scan)
    for (long long k = tid; k < c_hi - c_lo; k += WT) ctil[k] = 0;
  if (tid == 0) { s_bad[0] = 0; s_bad[1] = 0; }

  auto seg_of = [&](int s, int& rb, int& re) {
    rb = (s == 0) ? off0 : 0;
    re = (s == nseg - 1) ? (int)(c_hi - (long long)jb * D) : D;
  };

  // Emission values of the fold's step, loaded ahead: emw holds step t+1
  // while step t runs; thread s (< nseg) keeps step t+2's value and step
  // t+3's observation in registers.
  double em_pf = 0.0;
  int ob_pf = 0;
  if (tid < nseg) {
    const int j = ja + tid;
    if (2 < T) emw[tid] = m.em[(size_t)B.obs[2] * N + j];
    if (3 < T) em_pf = m.em[(size_t)B.obs[3] * N + j];
    if (4 < T) ob_pf = B.obs[4];
  }
  worker_sync_all<WT>();

  int r0 = 0;  // (t-1) % D
  int a3 = 1;  // t % 3: the buffer of E_t
  if (is_scan) {
    for (long long t = 1; t < T; ++t) {
      const int tau = (int)(t < D ? t : D);
      const long long t1 = t + 1;
      int r0n = r0 + 1;  // t % D: the slot that enters at step t+1 (d = 0 then)
      if (r0n == D) r0n = 0;
      const int an3 = a3 == 2 ? 0 : a3 + 1;  // (t+1) % 3
      if (tid < nseg) {
        if (t + 2 < T) emw[(int)((t + 2) & 1) * P.max_seg + tid] = em_pf;
        if (t + 3 < T) em_pf = m.em[(size_t)ob_pf * N + ja + tid];
        if (t + 4 < T) ob_pf = B.obs[t + 4];
      }

      // Phase 1: fixed-point scan over d in [L, tau), fused with the exact
      // window folds of step t+1 into the next buffer (src/hsmm.cu:298-310):
      // E_{t+1}[d] = E_t[d-1] + em_{t+1}, E_{t+1}[0] = 0 + em_{t+1}.  The FP64
      // adds overlap the integer scan.
      const bool fold = (t1 < T) && (t1 > D + 1);
      Top2* redb = red + (int)(t & 1) * P.max_seg * NW;
      for (int s = 0; s < nseg; ++s) {
        int rb, re;
        seg_of(s, rb, re);
        const long long* ct = ctil + s * D - off0;
        const long long* q = qd + s * D;
        const double* ac = accb + a3 * accs + s * D - off0;
        double* an = accb + an3 * accs + s * D - off0;
        const double em1 = fold ? emw[(int)(t1 & 1) * P.max_seg + s] : 0.0;
        Top2 tb, tc;  // two independent chains, merged after the loop
        tb.init();
        tc.init();
        if (qd_in_smem && tau == D) {
          // every d < D is in range; d < L is masked in the table
          int r = rb + tid;
#pragma unroll 2
          for (; r + WT < re; r += 2 * WT) {
            int d = r0 - r;
            if (d < 0) d += D;
            int d2 = d - WT;
            if (d2 < 0) d2 += D;
            const long long v0 = ct[r] + q[d], v1 = ct[r + WT] + q[d2];
            tb.push(v0, d);
            tc.push(v1, d2);
            if (fold) {
              an[r] = ((r == r0n) ? 0.0 : ac[r]) + em1;
              an[r + WT] = ((r + WT == r0n) ? 0.0 : ac[r + WT]) + em1;
            }
          }
          if (r < re) {
            int d = r0 - r;
            if (d < 0) d += D;
            tb.push(ct[r] + q[d], d);
            if (fold) an[r] = ((r == r0n) ? 0.0 : ac[r]) + em1;
          }
        } else {
#pragma unroll 4
          for (int r = rb + tid; r < re; r += WT) {
            int d = r0 - r;
            if (d < 0) d += D;
            if (d >= L && d < tau) tb.push(ct[r] + q[d], d);
            if (fold) an[r] = ((r == r0n) ? 0.0 : ac[r]) + em1;
          }
        }
        tb.merge(tc.b1, tc.x1, tc.b2);
        tb.warp_reduce();
        if (lane == 0) redb[s * NW + warp] = tb;
      }
      // Phase 2c: at t+1 = D+1 the first fold starts from the reference's
      // newest-first sums of step D: E_{D+1}[d] = E_D[d-1] + em_{D+1}.
      if (t1 < T && t1 == D + 1) {
        const int ot1 = B.obs[t1];
        for (int s = 0; s < nseg; ++s) {
          int rb, re;
          seg_of(s, rb, re);
          const int j = ja + s;
          const double em1 = m.em[(size_t)ot1 * N + j];
          double* an = accb + an3 * accs + s * D - off0;
          for (int r = rb + tid; r < re; r += WT) {
            int d = r0n - r;
            if (d < 0) d += D;
            const double base = (d == 0) ? 0.0 : early_window(m, B.ck, P.M, B.obs, D, d - 1, j);
            an[r] = base + em1;
          }
        }
      }
      worker_sync_all<WT>();  // phase 1 of step t done; the service work of step t-1 done
      if (*(volatile int*)&s_bad[(t - 1) & 1]) break;
      r0 = r0n;
      a3 = an3;
    }
  } else {
    for (long long t = 1; t < T; ++t) {
      const int tau = (int)(t < D ? t : D);
      int r0n = r0 + 1;
      if (r0n == D) r0n = 0;
      const int an3 = a3 == 2 ? 0 : a3 + 1;
      worker_sync_all<WT>();
      if (*(volatile int*)&s_bad[(t - 1) & 1]) break;
      if (warp == NW) {
        // Certify warp: the exact winner of each segment at step t, from the
        // scan's best and runner-up; lanes in groups of NW, a group per
        // segment, 32/NW segments at a time.
        const Top2* redb = red + (int)(t & 1) * P.max_seg * NW;
        const double* ac = accb + a3 * accs;  // E_t
        const unsigned prow = (unsigned)t & (PART_RING - 1);
        constexpr int GPW = 32 / NW;
        const int grp = lane / NW, gi = lane % NW;
        for (int s0 = 0; s0 < nseg; s0 += GPW) {
          const int s = s0 + grp;
          const bool sv = s < nseg;
          Top2 tb;
          tb.init();
          if (sv) tb = redb[s * NW + gi];
#pragma unroll
          for (int o = NW / 2; o > 0; o >>= 1) {
            const long long ob1 = __shfl_xor_sync(0xffffffffu, tb.b1, o);
            const long long ob2 = __shfl_xor_sync(0xffffffffu, tb.b2, o);
            const int ox1 = __shfl_xor_sync(0xffffffffu, tb.x1, o);
            tb.merge(ob1, ox1, ob2);
          }
          ExactBest eb;
          eb.init();
          bool amb = false;
          if (sv && gi == 0 && tb.x1 != IDX_NONE) {
            const int d1 = tb.x1;
            int r1 = r0 - d1;
            if (r1 < 0) r1 += D;
            const int c1 = s * D + r1 - off0;
            const unsigned short it = itil[c1];
            amb = (it & 0x8000) || ((tb.b1 - tb.b2) <= m.margin);
            if (!amb) {
              const int i1 = it & 0x7fff;
              const double e = (t > D) ? ac[c1] : early_window(m, B.ck, P.M, B.obs, t, d1, ja + s);
              eb.set((e + dsel[c1]) + (tr[s * N + i1] + dur[s * D + d1]), d1, i1);
            }
          }
          // Ambiguous segments: the whole warp re-scores every candidate
          // inside the margin exactly, one segment at a time.
          unsigned am = __ballot_sync(0xffffffffu, amb);
          while (am) {
            const int src = __ffs(am) - 1;
            am &= am - 1;
            const int sa = s0 + src / NW;
            const int j = ja + sa;
            const long long thr = __shfl_sync(0xffffffffu, tb.b1, src) - m.margin;
            int rb, re;
            seg_of(sa, rb, re);
            ExactBest ea;
            ea.init();
            bool ok = true;
            for (int r = rb + lane; r < re; r += 32) {
              int d = r0 - r;
              if (d < 0) d += D;
              if (d < L || d >= tau) continue;
              const int c = sa * D + r - off0;
              if (ctil[c] + qd[sa * D + d] < thr) continue;
              const double e = (t > D) ? ac[c] : early_window(m, B.ck, P.M, B.obs, t, d, j);
              const double du = dur[sa * D + d];
              for (int i = 0; i < N && ok; ++i) {
                double dv;
                ok = load_dstar(B, P, N, t - 1 - d, i, dv);
                if (ok) ea.offer((e + dv) + (tr[sa * N + i] + du), d, i);
              }
            }
            ea.warp_reduce();
            if (!__all_sync(0xffffffffu, ok)) {
              if (lane == 0) {
                grid_fail(B, TV_ETIMEOUT_DEV, SITE_WORKER_RESCORE);
                s_bad[t & 1] = 1;
              }
            }
            if (lane == src) eb = ea;
          }
          if (sv && gi == 0) send_partial(B, P, (unsigned)t, prow, seg0 + s, eb);
        }
      } else if (lane < nseg && t + 2 < T && t + 1 - L >= 0) {
        // Intake warp, one lane per segment: the slot s' = t+1-L, which
        // enters the scan at step t+2.  Lane 0 waits for the slot message
        // even when the slot is not its own: that is the flow control that
        // keeps a worker at most L-2 steps ahead of the head (its partials
        // ring holds PART_RING steps).
        const long long sp = t + 1 - L;
        int rn = r0 + 2 - L;  // sp % D
        if (rn < 0) rn += D;
        int rb, re;
        seg_of(lane, rb, re);
        const unsigned tag = (unsigned)(sp + 1);
        const unsigned long long* msg =
            B.slot_msg + ((size_t)((unsigned)sp & (SLOT_RING - 1)) * N + ja + lane) * SLOT_WORDS;
        const bool mine = rn >= rb && rn < re;
        if (mine || lane == 0) {
          unsigned long long cbits, dbits;
          unsigned ibits;
          if (!slot_load(msg, tag, cbits, dbits, ibits, B.abort_flag, P.timeout)) {
            grid_fail(B, TV_ETIMEOUT_DEV, SITE_WORKER_SLOT);
            s_bad[t & 1] = 1;
          } else if (mine) {
            const int c = lane * D + rn - off0;
            ctil[c] = (long long)cbits;
            dsel[c] = __longlong_as_double((long long)dbits);
            itil[c] = (unsigned short)(ibits & 0xffff);
          }
        }
      }
      r0 = r0n;
      a3 = an3;
    }
  }
  worker_sync_all<WT>();  // the service work of the last step is done
  if (s_bad[0] | s_bad[1]) return;
  if (!is_scan) return;

  // Tail at t = T-1: exhaustive exact scan of the worker's cells with the
  // survival function (src/hsmm.cu:101-137), one partial per segment.
  {
    const long long t = T - 1;
    const int tau = (int)(t < D ? t : D);
    const int rt = t >= 1 ? (int)((t - 1) % D) : 0;
    const double* ac = accb + (size_t)(t % 3) * accs;  // E_{T-1}
    for (int s = 0; s < nseg; ++s) {
      int rb, re;
      seg_of(s, rb, re);
      const int j = ja + s;
      ExactBest eb;
      eb.init();
      bool ok = true;
      for (int r = rb + tid; r < re && ok; r += WT) {
        int d = rt - r;
        if (d < 0) d += D;
        if (d < L || d >= tau) continue;
        const int c = s * D + r - off0;
        const double E = (t > D) ? ac[c] : early_window(m, B.ck, P.M, B.obs, t, d, j);
        const double e = E + m.survT[(size_t)j * D + d];
        for (int i = 0; i < N && ok; ++i) {
          double dv;
          ok = load_dstar(B, P, N, t - 1 - d, i, dv);
          if (ok) eb.offer((e + dv) + tr[s * N + i], d, i);
        }
      }
      if (!ok) {
        grid_fail(B, TV_ETIMEOUT_DEV, SITE_WORKER_TAIL);
        s_bad[0] = 1;
      }
      eb = worker_reduce_exact<WT>(eb, ered);
      if (s_bad[0]) return;
      if (tid == 0) send_partial(B, P, (unsigned)T, (unsigned)T & (PART_RING - 1), seg0 + s, eb);
    }
  }
}

// ---------------------------------------------------------------------------
// Head CTA
//
// The serial critical path of a step is: delta[t-1] final -> B[t-1][j] =
// max_i(trans[j][i] + delta[t-1][i]) for every j -> the d = 0 candidate ->
// merge -> delta[t].  Only that chain runs in the critical lanes, one per
// state:
//   * the matvec in packed int32: coarse score << 7 | (127 - i), so one
//     integer max yields the value and the lowest index; a second warp per 32
//     states scans the upper half of i and hands its best and runner-up over;
//     the runner-up gap is certified against a coarse margin, else a fine
//     int64 pass decides;
//   * then, in the same lane (no other state's slot is needed), the dense
//     phase: the d = 0 candidate's fixed-point score W0 against Wtop, the best
//     fixed-point score over d >= 1 that the helpers prepared with the exact
//     winner among d >= 1.  When W0 trails Wtop by more than the certified
//     margin, delta[t] is that winner; otherwise the d = 0 score, computed
//     exactly (two dependent FP64 adds) ahead of the test, is compared.
// FP64 instructions cost the same pipe time whatever the number of active
// lanes, so exact scores are computed one lane per state in dense warps.
// The helpers prepare the next steps meanwhile: the intake of the workers'
// partial winners (loaded a step ahead), window sums (bulk-copied three steps
// ahead from a table built before the launch), and in two alternating groups
// the candidates d = 1..L-1 in fixed point, certification, the exact score of
// the winner when it is one of them, and all global stores.  Named barriers
// hand slot t-1 from the critical lanes to the helpers and the prepared
// winner back.
// ---------------------------------------------------------------------------
constexpr int HWR = 4;  // rows of window sums kept by the head: steps t .. t+3

// Named barriers of the head CTA (the CTA-wide barrier 0 is used only while
// every thread is alive; threads without a role leave before the steps).
// Non-aligned forms: they count threads, so a warp whose lanes took different
// branches may arrive lane by lane.
enum { BAR_STEP = 1, BAR_SLOT0 = 2, BAR_PW0 = 4, BAR_SLOT1 = 5, BAR_PW1 = 6, BAR_PRE0 = 7, BAR_PRE1 = 8,
       BAR_END = 9, BAR_PAIR0 = 10 };  // BAR_PAIR0 + k: the matvec halves of state group k (k < 4)
__device__ __forceinline__ void named_sync(int id, int count) {
  asm volatile("barrier.sync %0, %1;" ::"r"(id), "r"(count) : "memory");
}
__device__ __forceinline__ void named_arrive(int id, int count) {
  asm volatile("barrier.arrive %0, %1;" ::"r"(id), "r"(count) : "memory");
}

// One-shot bulk copies (global -> shared) completed on an mbarrier: the
// issuing thread announces the byte count, the copy engine moves the bytes
// and completes the barrier's phase; a waiter polls the phase parity.
__device__ __forceinline__ void mbar_init(unsigned long long* bar, unsigned count) {
  const unsigned a = (unsigned)__cvta_generic_to_shared(bar);
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(a), "r"(count) : "memory");
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}
__device__ __forceinline__ void bulk_copy_g2s(void* dst, const void* src, unsigned bytes, unsigned long long* bar) {
  const unsigned d = (unsigned)__cvta_generic_to_shared(dst);
  const unsigned a = (unsigned)__cvta_generic_to_shared(bar);
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(a), "r"(bytes) : "memory");
  asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];"
               ::"r"(d), "l"(src), "r"(bytes), "r"(a) : "memory");
}
__device__ __forceinline__ bool mbar_test(unsigned long long* bar, unsigned parity) {
  const unsigned a = (unsigned)__cvta_generic_to_shared(bar);
  unsigned ok;
  asm volatile("{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}"
               : "=r"(ok) : "r"(a), "r"(parity) : "memory");
  return ok != 0;
}
// Waits (bounded) for the phase with the given parity to complete.
__device__ __forceinline__ bool mbar_wait(unsigned long long* bar, unsigned parity, long long limit) {
  if (mbar_test(bar, parity)) return true;
  const long long t0 = clock64();
  while (!mbar_test(bar, parity))
    if (clock64() - t0 > limit) return false;
  return true;
}

__device__ __forceinline__ int coarse_of(long long fine_minus_base, int sh) {
  long long v = fine_minus_base >> sh;  // arithmetic shift: floor
  v = v > COARSE_CLAMP ? COARSE_CLAMP : (v < -COARSE_CLAMP ? -COARSE_CLAMP : v);
  return (int)v;
}

// Packed coarse top-2: one max keeps the value and the lowest index.
__device__ __forceinline__ void packed_push(int p, int& b1, int& b2) {
  const int lo = min(b1, p);
  b1 = max(b1, p);
  b2 = max(b2, lo);
}


// A worker segment's exact winner, kept as its order key and its fixed-point
// value (the value of the segment's best candidate, to within half a unit),
// both computed by the worker.
__device__ __forceinline__ void take_partial(const TaggedMsg& pm, int k, long long* pwq, long long* pwk, int* pwd,
                                             int* pwi) {
  long long key, fx;
  unsigned di;
  msg_unpack(pm, key, fx, di);
  pwq[k] = fx;
  pwk[k] = key;
  pwd[k] = (int)(di >> 16);
  pwi[k] = (int)(di & 0xffff);
}

__device__ void grid_head(const ModelView& m, const GridParams& P, const GridBufs& B, unsigned char* sm) {
  constexpr int L = GRID_L;
  const int N = m.N, D = m.D, S = P.S, Np = P.Np;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const long long T = B.T;
  const long long margin = m.margin;
  // [N][Qs] packed coarse trans; the row stride Qs = Np + 4 puts the 16-byte
  // pieces that 8 consecutive states' lanes load together in 8 different
  // bank quads (Np/4 is even, Qs/4 odd)
  const int Qs = Np + 4;
  int* Qcp = (int*)(sm + P.h_qcp);
  long long* qtr_s = (long long*)(sm + P.h_qtr);      // [N][N] fine trans (when it fits)
  double* trh_s = (double*)(sm + P.h_trh);            // [N][N] exact trans (when it fits)
  const double* trh = P.trans_smem ? trh_s : m.trans;
  // fixed-point transition score: the shared copy, else quantised from the
  // exact table (the same rounding as the copy), else the global copy
  auto qtr_at = [&](int j, int i) -> long long {
    if (P.qtr_smem) return qtr_s[j * N + i];
    if (P.trans_smem) return quantize(trh_s[j * N + i], m.scale);
    return m.qtr[(size_t)j * N + i];
  };
  int* dqcp = (int*)(sm + P.h_dqcp);                  // [2][Np] packed coarse delta
  long long* dq = (long long*)(sm + P.h_dq);          // [2][N] fine delta
  long long* ptil = (long long*)(sm + P.h_ptil);      // [4][N] emission prefix P(t), row t % 4
  long long* basebuf = (long long*)(sm + P.h_base);   // [2] coarse base per step
  double* dstar_h = (double*)(sm + P.h_dstar);        // [L+1][N] exact delta
  long long* ctil_h = (long long*)(sm + P.h_ctil);    // [L][N]
  unsigned short* itil_h = (unsigned short*)(sm + P.h_itil);
  double* hwr = (double*)(sm + P.h_hwr);              // [HWR][L][N] window sums, row t % HWR
  long long* qd_h = (long long*)(sm + P.h_qd);        // [L][N] (consecutive states, consecutive banks)
  double* dur_h = (double*)(sm + P.h_dur);            // [L][N]
  long long* prek = (long long*)(sm + P.h_prek);      // [2][N] exact winner over d >= 1: order key
  int* pred = (int*)(sm + P.h_pred);
  int* prei = (int*)(sm + P.h_prei);
  long long* prew = (long long*)(sm + P.h_prew);      // [2][N] best fixed-point score over d >= 1
  long long* preq = (long long*)(sm + P.h_preq);      // [2][N] fixed-point value of the exact winner
  uint32_t* psirec = (uint32_t*)(sm + P.h_psirec);    // [4][N] back-pointer words, row t % 4
  long long* pwq = (long long*)(sm + P.h_pwq);        // [2][S] worker partials, by step parity
  long long* pwk = (long long*)(sm + P.h_pwk);
  int* pwd = (int*)(sm + P.h_pwd);
  int* pwi = (int*)(sm + P.h_pwi);
  double* tail = (double*)(sm + P.h_tail);
  // Failure flags: s_fail for the set-up and the tail; s_fb[t & 1] for an
  // intake failure at step t of the loops (1), or the intake's notice that
  // the loops end at step t-1 (2), read by every role at points where its
  // value for step t is settled, so that all roles leave at the same step.
  __shared__ int s_fail;
  __shared__ int s_fb[2];
  __shared__ __align__(8) unsigned long long s_hwbar;  // completion of the window-sum row copies
  const int sh = P.coarse_shift;
  // Roles, by thread range:
  //   [0, cs)               critical: one lane per state, the matvec of slot
  //                         t-1 and then the dense phase of delta[t]
  //   [cs, cs+csb)          (when split) the upper half of each matvec, a warp
  //                         per 32 states, handed over through shared memory
  //   [cs+csb, +2*st)       state helpers in two groups, one lane per state;
  //                         group g prepares step t+1 for the steps t of parity
  //                         g (certification and exact winner over d >= 1), then
  //                         stores step t-1's results and slot t-1's messages;
  //                         a group has two steps for its work, so its serial
  //                         chain overlaps the other's
  //   [cs+csb+2*st, nthr)   intake: the workers' partial winners (a lane takes
  //                         segments pk and pk + in), the emission prefix (one
  //                         lane per state), the window-sum copies and the coarse
  //                         base
  // Threads beyond these leave once the tables are set up.
  const int cs = P.cs_threads, st = P.st_threads, in = P.in_threads;
  const int csb = P.cs_split ? cs : 0;
  const int nthr = cs + csb + 2 * st + in;
  const bool is_cs = tid < cs;
  const bool is_csb = !is_cs && tid < cs + csb;
  const bool is_st = !is_cs && !is_csb && tid < cs + csb + 2 * st;
  const bool is_in = !is_cs && !is_csb && !is_st && tid < nthr;
  // the matvec's split point over i (a multiple of 8), and its upper half's
  // best and runner-up per state
  const int Nh = P.cs_split ? (Np / 16) * 8 : Np;
  int2* xch = (int2*)(sm + P.h_xch);
  const int sg = is_st ? (tid - cs - csb) / st : 0;    // state helper: group (parity of its steps)
  const int sj = is_st ? (tid - cs - csb) % st : 0;    // state helper: state
  const int pk = tid - cs - csb - 2 * st;              // intake: lane
  const bool has_sj = is_st && sj < N;
  const bool has_pk = is_in && pk < S;
  const bool has_pk2 = is_in && pk + in < S;
  const bool has_pj = is_in && pk < N;                 // in >= N: a lane per state too
  int k0 = 0, k1 = 0;
  if (has_sj) {
    k0 = B.seg_first[sj];
    k1 = k0 + B.seg_count[sj];
  }

  // ---- initial state (t = 0), all threads ----
  for (int k = tid; k < N * Np; k += blockDim.x) {
    const int jj = k / Np, i = k % Np;
    if (i < N) {
      const int c = coarse_of(m.qtr[(size_t)jj * N + i], sh);
      Qcp[jj * Qs + i] = c * 128 + (127 - i);
    } else {
      Qcp[jj * Qs + i] = INT_MIN;
    }
  }
  for (int k = tid; k < N * N; k += blockDim.x) {
    if (P.qtr_smem) qtr_s[k] = m.qtr[k];
    if (P.trans_smem) trh_s[k] = m.trans[k];
  }
  for (int k = tid; k < N * L; k += blockDim.x) {
    const int d = k / N, jj = k % N;
    qd_h[k] = m.qdurT[(size_t)jj * D + d];
    dur_h[k] = m.durT[(size_t)jj * D + d];
  }
  for (int k = tid; k < 2 * Np; k += blockDim.x) dqcp[k] = 0;
  for (int jj = tid; jj < N; jj += blockDim.x) {
    const double d0 = B.dinit[jj];
    dstar_h[jj] = d0;
    tagged64_store(B.dstar + (size_t)jj * 2, 1u, (unsigned long long)__double_as_longlong(d0));
    dq[jj] = fixed_from_double(d0, P.qf);
    const long long p0 = m.qem[(size_t)B.obs[0] * N + jj];
    ptil[jj] = p0;                                                        // P(0)
    if (T > 1) ptil[N + jj] = p0 + m.qem[(size_t)B.obs[1] * N + jj];  // P(1)
    B.psi[jj] = pack_psi(0, 0);
  }
  for (int k = tid; k < HWR * L * N; k += blockDim.x)  // window sums of steps 0..3
    if (k / (L * N) < T) hwr[k] = B.hwin[k];
  if (tid == 0) {
    s_fail = 0;
    s_fb[0] = 0;
    s_fb[1] = 0;
    mbar_init(&s_hwbar, 1);
  }
  __syncthreads();
  if (warp == 0) {
    long long mx = LLONG_MIN;
    for (int jj = lane; jj < N; jj += 32) mx = max(mx, dq[jj]);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) mx = max(mx, __shfl_xor_sync(0xffffffffu, mx, o));
    if (lane == 0) { basebuf[0] = mx; basebuf[1] = mx; }
  }
  __syncthreads();
  for (int jj = tid; jj < N; jj += blockDim.x) dqcp[jj] = coarse_of(dq[jj] - basebuf[0], sh) * 128;
  // worker partials of step 1 (all empty: no d >= L yet) into buffer 1, and
  // the prefetch of step 2
  TaggedMsg pm, pm2;
  auto intake_one = [&](int seg, TaggedMsg& msg, long long step, int site, int* flag) {
    const unsigned long long* src = B.part + ((size_t)((unsigned)step & (PART_RING - 1)) * S + seg) * MSG_WORDS;
    if (!msg_wait(src, (unsigned)step, msg, B.abort_flag, P.timeout)) {
      grid_fail(B, TV_ETIMEOUT_DEV, site);
      *flag = 1;
    } else {
      const int pb = (int)(step & 1) * S;
      take_partial(msg, seg, pwq + pb, pwk + pb, pwd + pb, pwi + pb);
    }
  };
  if (T > 1) {
    if (has_pk) {
      msg_load(B.part + ((size_t)(1 & (PART_RING - 1)) * S + pk) * MSG_WORDS, pm);
      intake_one(pk, pm, 1, SITE_HEAD_PARTIAL, &s_fail);
      if (T > 2) msg_load(B.part + ((size_t)(2 & (PART_RING - 1)) * S + pk) * MSG_WORDS, pm);
    }
    if (has_pk2) {
      msg_load(B.part + ((size_t)(1 & (PART_RING - 1)) * S + pk + in) * MSG_WORDS, pm2);
      intake_one(pk + in, pm2, 1, SITE_HEAD_PARTIAL, &s_fail);
      if (T > 2) msg_load(B.part + ((size_t)(2 & (PART_RING - 1)) * S + pk + in) * MSG_WORDS, pm2);
    }
  }
  __syncthreads();
  if (s_fail) return;
  for (int jj = tid; jj < N; jj += blockDim.x) {
    const int a = B.seg_first[jj], b = a + B.seg_count[jj];
    const long long p1 = ptil[N + jj];
    const long long* pq1 = pwq + S;
    const long long* pk1 = pwk + S;
    const int* pd1 = pwd + S;
    const int* pi1 = pwi + S;
    long long W = QNEG;
    for (int k = a; k < b; ++k)
      if (pd1[k] != EMPTY_D) W = max(W, pq1[k] - p1);
    ExactBest eb;
    eb.init();
    for (int k = a; k < b; ++k)
      if (pd1[k] != EMPTY_D && pq1[k] - p1 >= W - margin) eb.offer_key(pk1[k], pd1[k], pi1[k]);
    prew[(1 & 1) * N + jj] = W;
    prek[(1 & 1) * N + jj] = eb.k;
    pred[(1 & 1) * N + jj] = eb.d;
    prei[(1 & 1) * N + jj] = eb.i;
    preq[(1 & 1) * N + jj] = eb.d != IDX_NONE ? fixed_from_double(eb.value(), P.qf) : 0;
  }
  __syncthreads();
  if (tid >= nthr) return;  // no role in the steps

  // Register pipelines: an intake lane keeps the partial messages of step t+2
  // (pm, pm2) and, for its state, the prefix term of step t+2 and the
  // observation of step t+3; a dense critical lane the initialisation score of
  // step t+1.
  long long qe_pf = 0;
  int ob_q = 0;
  if (has_pj) {
    if (2 < T) qe_pf = m.qem[(size_t)B.obs[2] * N + pk];
    if (3 < T) ob_q = B.obs[3];
  }
  double di_cur = 0.0;  // initialisation score of step t, state tid (dense critical lanes)
  if (tid < N && 1 < D) di_cur = __ldcg(B.dinit + (size_t)1 * N + tid);

  int drow_prev = 0;  // (t-1) % (L+1): row of delta[t-1] in dstar_h
  if (is_cs) {
    // ================= critical lanes: every step, one lane per state =================
    // The lane of state j computes slot t-1 of j (the matvec) and then delta[t]
    // of j (the dense phase): neither needs another state's slot, so no barrier
    // separates them and the slot stays in registers.
    const int j = tid;
    for (long long t = 1; t < T; ++t) {
      const int cur = (int)(t & 1), prv = cur ^ 1;
      const int drow = drow_prev + 1 == L + 1 ? 0 : drow_prev + 1;  // t % (L+1)
      const int hrow = (int)((t - 1) & (L - 1));                      // slot t-1 in ctil_h
      double di_next = 0.0;
      if (j < N && t + 1 < D) di_next = __ldcg(B.dinit + (size_t)(t + 1) * N + j);
      long long cv = 0;
      int ifine = 0;
      bool amb = false;
      // packed coarse matvec over i for slot t-1: coarse score << 7 |
      // (127 - i), so one integer max gives the value and the lowest index;
      // two independent chains of (best, runner-up)
      int b1 = INT_MIN, b2 = INT_MIN;
      if (j < N) {
        int c1 = INT_MIN, c2 = INT_MIN;
        const int* qrow = Qcp + j * Qs;
        const int* dv = dqcp + prv * Np;
#pragma unroll 2
        for (int i4 = 0; i4 < Nh; i4 += 8) {
          const int4 a0 = *reinterpret_cast<const int4*>(qrow + i4);
          const int4 d0 = *reinterpret_cast<const int4*>(dv + i4);
          const int4 a1 = *reinterpret_cast<const int4*>(qrow + i4 + 4);
          const int4 d1 = *reinterpret_cast<const int4*>(dv + i4 + 4);
          packed_push(a0.x + d0.x, b1, b2);
          packed_push(a1.x + d1.x, c1, c2);
          packed_push(a0.y + d0.y, b1, b2);
          packed_push(a1.y + d1.y, c1, c2);
          packed_push(a0.z + d0.z, b1, b2);
          packed_push(a1.z + d1.z, c1, c2);
          packed_push(a0.w + d0.w, b1, b2);
          packed_push(a1.w + d1.w, c1, c2);
        }
        const int lo = min(b1, c1);
        b1 = max(b1, c1);
        b2 = max(max(b2, c2), lo);
      }
      if (P.cs_split) named_sync(BAR_PAIR0 + (tid >> 5), 64);  // the upper half of this warp's states is in
      if (j < N) {
        if (P.cs_split) {
          const int2 o = xch[j];
          const int lo = min(b1, o.x);
          b1 = max(b1, o.x);
          b2 = max(max(b2, o.y), lo);
        }
        ifine = 127 - (b1 & 127);
        amb = ((b1 >> 7) - (b2 >> 7)) <= P.coarse_margin;
        long long bfine;
        if (!amb) {
          bfine = qtr_at(j, ifine) + dq[prv * N + ifine];
        } else {
          // fine int64 pass decides (and certifies with the fine margin)
          Top2 tb;
          tb.init();
          const long long* qrow_f = P.qtr_smem ? qtr_s + (size_t)j * N : m.qtr + (size_t)j * N;
          for (int i = 0; i < N; ++i) tb.push(qrow_f[i] + dq[prv * N + i], i);
          ifine = tb.x1;
          bfine = tb.b1;
          amb = (tb.b1 - tb.b2) <= margin;
        }
        cv = bfine - ptil[(int)((t - 1) & 3) * N + j];  // relative to the emission prefix P(t-1)
        ctil_h[hrow * N + j] = cv;
        itil_h[hrow * N + j] = (unsigned short)(ifine | (amb ? 0x8000 : 0));
      }
      // slot t-1 ready for the group of step t (its d = 1) and the group of
      // step t+1 (its d >= 2)
      named_arrive(cur ? BAR_SLOT1 : BAR_SLOT0, t + 1 < T ? cs + 2 * st : cs + st);
      // the winner over d >= 1 of step t, prepared by the group of step t-1
      if (t >= 2) named_sync(prv ? BAR_PRE1 : BAR_PRE0, cs + st);
      if (j < N) {
        // Dense phase: the d = 0 candidate's fixed-point score W0 against
        // Wtop, the best over d >= 1 with its exact winner; the exact d = 0
        // score of the certified argmax over i is computed before it is known
        // to be needed.
        const long long W0 = cv + qd_h[j];
        const long long Wt = prew[cur * N + j];
        const long long pk0 = prek[cur * N + j];
        const int pd0 = pred[cur * N + j], pi0 = prei[cur * N + j];
        const long long pq0 = preq[cur * N + j];
        const double e0 = hwr[(int)(t & (HWR - 1)) * L * N + j];
        const double du0 = dur_h[j];
        // src/hsmm.cu:341-346 with E_t[0]
        const double V0 = (e0 + dstar_h[drow_prev * N + ifine]) + (trh[(size_t)j * N + ifine] + du0);
        const long long q0 = fixed_from_double(V0, P.qf);
        long long kk = pk0, fq = pq0;
        int dd = pd0, ii = pi0;
        if (W0 >= Wt - margin) {
          ExactBest eb;
          if (!amb) {
            eb.set(V0, 0, ifine);
          } else {
            eb.init();
            const double* row = dstar_h + drow_prev * N;
            const double* trj = trh + (size_t)j * N;
            for (int i = 0; i < N; ++i) eb.offer((e0 + row[i]) + (trj[i] + du0), 0, i);
          }
          if (W0 <= Wt + margin) eb.offer_key(pk0, pd0, pi0);
          kk = eb.k;
          dd = eb.d;
          ii = eb.i;
          if (dd == 0) fq = amb ? fixed_from_double(eb.value(), P.qf) : q0;
        }
        double fin = key_value(kk);
        uint32_t wv = pack_psi(dd, ii);
        // t < D: the induction result replaces the initialisation score only
        // when strictly larger (src/hsmm.cu:353-358).
        if (t < D && !(kk > order_key(di_cur))) {
          fin = di_cur;
          wv = pack_psi((int)t, 0);
          fq = fixed_from_double(fin, P.qf);
        }
        dstar_h[drow * N + j] = fin;
        dq[cur * N + j] = fq;
        dqcp[cur * Np + j] = coarse_of(fq - basebuf[cur], sh) * 128;
        psirec[(int)(t & 3) * N + j] = wv;
      }
      di_cur = di_next;
      drow_prev = drow;
      named_sync(BAR_STEP, cs + csb + in);
      if (*(volatile int*)&s_fb[cur]) break;  // the intake failed at this step
    }
  } else if (is_csb) {
    // ============ upper half of the matvec: every step, one lane per state ============
    const int jb = tid - cs;
    for (long long t = 1; t < T; ++t) {
      const int cur = (int)(t & 1), prv = cur ^ 1;
      if (jb < N) {
        int b1 = INT_MIN, b2 = INT_MIN, c1 = INT_MIN, c2 = INT_MIN;
        const int* qrow = Qcp + jb * Qs;
        const int* dv = dqcp + prv * Np;
#pragma unroll 2
        for (int i4 = Nh; i4 < Np; i4 += 8) {
          const int4 a0 = *reinterpret_cast<const int4*>(qrow + i4);
          const int4 d0 = *reinterpret_cast<const int4*>(dv + i4);
          const int4 a1 = *reinterpret_cast<const int4*>(qrow + i4 + 4);
          const int4 d1 = *reinterpret_cast<const int4*>(dv + i4 + 4);
          packed_push(a0.x + d0.x, b1, b2);
          packed_push(a1.x + d1.x, c1, c2);
          packed_push(a0.y + d0.y, b1, b2);
          packed_push(a1.y + d1.y, c1, c2);
          packed_push(a0.z + d0.z, b1, b2);
          packed_push(a1.z + d1.z, c1, c2);
          packed_push(a0.w + d0.w, b1, b2);
          packed_push(a1.w + d1.w, c1, c2);
        }
        const int lo = min(b1, c1);
        xch[jb] = make_int2(max(b1, c1), max(max(b2, c2), lo));
      }
      named_arrive(BAR_PAIR0 + (jb >> 5), 64);
      named_sync(BAR_STEP, cs + csb + in);
      if (*(volatile int*)&s_fb[cur]) break;  // the intake failed at this step
    }
  } else if (is_st) {
    // ============ state helpers: group sg takes the steps of parity sg ============
    for (long long t = sg ? 1 : 2; t < T; t += 2) {
      const long long t1 = t + 1;
      const bool next = t1 < T;
      const int ti = (int)t;
      const int bw = (int)(t1 & 1) * S;  // partial buffer of step t+1
      const int own_cnt = next ? cs + 2 * st : cs + st;  // slot t-1 is also awaited by the group of step t+1
      // Every candidate d >= 1 of step t+1 in fixed point: d = 1..L-1 here
      // (slots t-d), d >= L as the workers' winners, whose fixed-point scores
      // are their values minus the prefix P(t+1).  The slots t-2..t-L+1 are in
      // once the critical lanes published slot t-2 (their step t-1): their
      // best and runner-up come first, before the partials arrive.  Only d = 1
      // needs slot t-1, which the critical lanes compute meanwhile.
      if (t >= 2) named_sync(((t - 1) & 1) ? BAR_SLOT1 : BAR_SLOT0, cs + 2 * st);
      const int tau1 = (int)(t1 < D ? t1 : D);
      const int hl1 = tau1 < L ? tau1 : L;
      long long Wd[L];
      unsigned short itd[L];
      long long Wh = QNEG, W2 = QNEG;
      int dh = 0, ih = 0, hamb = 0;
      if (has_sj && next) {
#pragma unroll
        for (int d = 2; d < L; ++d) {
          const int row = (ti - d) & (L - 1);
          Wd[d] = d < hl1 ? ctil_h[row * N + sj] + qd_h[d * N + sj] : QNEG;
          itd[d] = itil_h[row * N + sj];
        }
#pragma unroll
        for (int d = 2; d < L; ++d) {
          W2 = max(W2, min(Wh, Wd[d]));
          if (Wd[d] > Wh) {
            Wh = Wd[d];
            dh = d;
            ih = itd[d] & 0x7fff;
            hamb = itd[d] & 0x8000;
          }
        }
      }
      named_sync(sg ? BAR_PW1 : BAR_PW0, st + in);  // partials of step t+1, P(t+1), window sums of t+1 are in
      const int fb = *(volatile int*)&s_fb[sg];
      if (fb == 2) break;  // the loops ended at step t-1
      if (fb == 1) {       // the intake failed at this step: the critical warps finish it, then leave
        named_sync(sg ? BAR_SLOT1 : BAR_SLOT0, own_cnt);
        break;
      }
      // the exact winner among the candidates within the margin of the best
      // over d >= 2, with the exact score of the best short candidate computed
      // before it is known to be needed
      long long Wr = QNEG;
      ExactBest er;
      er.init();
      long long qr = 0;
      if (has_sj && next) {
        const long long p1 = ptil[(int)(t1 & 3) * N + sj];
        double Vh = 0.0;
        long long qh = 0;
        if (dh > 0) {
          const int dr = (ti - dh) % (L + 1);  // row of delta[t-dh]
          const double e = hwr[((int)(t1 & (HWR - 1)) * L + dh) * N + sj];
          Vh = (e + dstar_h[dr * N + ih]) + (trh[(size_t)sj * N + ih] + dur_h[dh * N + sj]);
          qh = fixed_from_double(Vh, P.qf);
        }
        Wr = Wh;
        for (int k = k0; k < k1; ++k)
          if (pwd[bw + k] != EMPTY_D) Wr = max(Wr, pwq[bw + k] - p1);
        const long long thr = Wr - margin;
        for (int k = k0; k < k1; ++k)
          if (pwd[bw + k] != EMPTY_D && pwq[bw + k] - p1 >= thr &&
              er.better_key(pwk[bw + k], pwd[bw + k], pwi[bw + k])) {
            er.k = pwk[bw + k];
            er.d = pwd[bw + k];
            er.i = pwi[bw + k];
            qr = pwq[bw + k];
          }
        if (Wh >= thr) {
          if (W2 < thr && !hamb) {
            // one short candidate in the margin, argmax over i certified
            const long long kh = order_key(Vh);
            if (er.better_key(kh, dh, ih)) {
              er.k = kh;
              er.d = dh;
              er.i = ih;
              qr = qh;
            }
          } else {
            // several in the margin, or an ambiguous argmax over i (rare)
            for (int d = 2; d < hl1; ++d) {
              if (Wd[d] < thr) continue;
              const double e = hwr[((int)(t1 & (HWR - 1)) * L + d) * N + sj];
              const double du = dur_h[d * N + sj];
              const double* drw = dstar_h + ((ti - d) % (L + 1)) * N;
              const double* trj = trh + (size_t)sj * N;
              const unsigned short it = itd[d];
              if (!(it & 0x8000)) {
                const int i1 = it & 0x7fff;
                er.offer((e + drw[i1]) + (trj[i1] + du), d, i1);
              } else {
                for (int i = 0; i < N; ++i) er.offer((e + drw[i]) + (trj[i] + du), d, i);
              }
            }
            qr = er.d == IDX_NONE ? 0 : fixed_from_double(er.value(), P.qf);
          }
        }
      }
      named_sync(sg ? BAR_SLOT1 : BAR_SLOT0, own_cnt);  // the critical lanes published slot t-1
      const int hrow = (ti - 1) & (L - 1);               // slot t-1
      const int drw1 = (ti - 1) % (L + 1);               // row of delta[t-1]
      if (has_sj && next) {
        // d = 1 (slot t-1): merged exactly when it is within the margin of R
        const long long W1 = hl1 > 1 ? ctil_h[hrow * N + sj] + qd_h[N + sj] : QNEG;
        const unsigned short it1 = itil_h[hrow * N + sj];
        if (hl1 > 1 && W1 >= Wr - margin) {
          const double e = hwr[((int)(t1 & (HWR - 1)) * L + 1) * N + sj];
          const double du = dur_h[N + sj];
          const double* drw = dstar_h + drw1 * N;
          const double* trj = trh + (size_t)sj * N;
          if (!(it1 & 0x8000)) {
            const int i1 = it1 & 0x7fff;
            const double V1 = (e + drw[i1]) + (trj[i1] + du);
            const long long k1v = order_key(V1);
            if (er.better_key(k1v, 1, i1)) {
              er.k = k1v;
              er.d = 1;
              er.i = i1;
              qr = fixed_from_double(V1, P.qf);
            }
          } else {
            for (int i = 0; i < N; ++i) er.offer((e + drw[i]) + (trj[i] + du), 1, i);
            qr = er.d == IDX_NONE ? 0 : fixed_from_double(er.value(), P.qf);
          }
        }
        const int nx = (int)(t1 & 1);
        prew[nx * N + sj] = max(Wr, W1);
        prek[nx * N + sj] = er.k;
        pred[nx * N + sj] = er.d;
        prei[nx * N + sj] = er.i;
        preq[nx * N + sj] = qr;
      }
      if (next) named_arrive(sg ? BAR_PRE1 : BAR_PRE0, cs + st);
      // results of step t-1, off the critical path: the slot t-1 messages
      // for the workers (score, selected delta[t-1][i*], argmax word), the
      // back-pointers and delta[t-1] in the exact ring the workers read
      if (has_sj) {
        const unsigned tag = (unsigned)t;
        const unsigned short itv = itil_h[hrow * N + sj];
        unsigned long long* msg =
            B.slot_msg + ((size_t)((unsigned)(t - 1) & (SLOT_RING - 1)) * N + sj) * SLOT_WORDS;
        tagged64_store(msg, tag, (unsigned long long)ctil_h[hrow * N + sj]);
        tagged64_store(msg + 2, tag, (unsigned long long)__double_as_longlong(dstar_h[drw1 * N + (itv & 0x7fff)]));
        st_relaxed_u64(msg + 4, ((unsigned long long)tag << 32) | itv);
        if (t >= 2) {
          B.psi[(size_t)(t - 1) * N + sj] = psirec[((ti - 1) & 3) * N + sj];
          tagged64_store(B.dstar + ((size_t)((ti - 1) % P.Rd) * N + sj) * 2, tag,
                         (unsigned long long)__double_as_longlong(dstar_h[drw1 * N + sj]));
        }
      }
    }
  } else {
    // ============ intake: every step ============
    long long last_copy = -1;  // a window-sum copy issued and not yet waited for
    for (long long t = 1; t < T; ++t) {
      const long long t1 = t + 1;
      const bool next = t1 < T;
      const int cur = (int)(t & 1), prv = cur ^ 1;
      // worker partials of step t+1 (loaded during the previous step) into buffer (t+1) & 1
      if (next) {
        if (has_pk) intake_one(pk, pm, t1, SITE_HEAD_PARTIAL, &s_fb[cur]);
        if (has_pk2) intake_one(pk + in, pm2, t1, SITE_HEAD_PARTIAL, &s_fb[cur]);
        if (has_pj) ptil[(int)(t1 & 3) * N + pk] = ptil[(int)(t & 3) * N + pk] + qe_pf;  // P(t+1)
      }
      // the window sums of step t+2 (copied during the previous step) are in
      // before the group of step t+1 is released
      if (pk == 0 && t >= 2 && t + 2 < T) {
        if (mbar_wait(&s_hwbar, (unsigned)(t & 1), P.copy_timeout)) {
          last_copy = -1;
        } else {
          grid_fail(B, TV_ETIMEOUT_DEV, SITE_HEAD_COPY);
          s_fb[cur] = 1;
        }
      }
      named_arrive(cur ? BAR_PW1 : BAR_PW0, st + in);
      // loads for the next step, issued once the state helpers are released:
      // the partials of step t+2, the prefix term of step t+2, the
      // observation of step t+3
      if (next) {
        if (has_pk && t1 + 1 < T)
          msg_load(B.part + ((size_t)((unsigned)(t1 + 1) & (PART_RING - 1)) * S + pk) * MSG_WORDS, pm);
        if (has_pk2 && t1 + 1 < T)
          msg_load(B.part + ((size_t)((unsigned)(t1 + 1) & (PART_RING - 1)) * S + pk + in) * MSG_WORDS, pm2);
        if (has_pj) {
          if (t + 2 < T) qe_pf = m.qem[(size_t)ob_q * N + pk];
          if (t + 3 < T) ob_q = B.obs[t + 3];
        }
      }
      // window sums of step t+3 into the ring: one bulk copy
      if (pk == 0 && t + 3 < T) {
        bulk_copy_g2s(hwr + (int)((t + 3) & (HWR - 1)) * L * N, B.hwin + (size_t)(t + 3) * L * N,
                      (unsigned)(L * N * sizeof(double)), &s_hwbar);
        last_copy = t - 1;  // the copy's index: it completes the barrier's phase t-1
      }
      // coarse base of step t+1: max_i delta[t-1] (the first intake warp)
      if (pk < 32) {
        long long mx = LLONG_MIN;
        for (int i = pk; i < N; i += 32) mx = max(mx, dq[prv * N + i]);
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) mx = max(mx, __shfl_xor_sync(0xffffffffu, mx, o));
        if (pk == 0) basebuf[cur ^ 1] = mx;
      }
      named_sync(BAR_STEP, cs + csb + in);
      if (*(volatile int*)&s_fb[cur]) {
        // the intake failed at this step: the group of step t+1 waits for its
        // partials; wake it with the notice that the loops end here
        s_fb[prv] = 2;
        named_arrive(prv ? BAR_PW1 : BAR_PW0, st + in);
        break;
      }
    }
    // a copy still in flight after an early exit
    if (pk == 0 && last_copy >= 0 && !mbar_wait(&s_hwbar, (unsigned)(last_copy & 1), P.copy_timeout)) s_fb[0] = 1;
  }
  named_sync(BAR_END, nthr);
  if (s_fb[0] | s_fb[1]) return;

  // Tail at t = T-1 (src/hsmm.cu:101-137).
  {
    const long long t = T - 1;
    const int tau = (int)(t < D ? t : D);
    const int hl = tau < L ? tau : L;
    if (has_pk) {
      msg_load(B.part + ((size_t)((unsigned)T & (PART_RING - 1)) * S + pk) * MSG_WORDS, pm);
      intake_one(pk, pm, T, SITE_HEAD_TAIL, &s_fail);
    }
    if (has_pk2) {
      msg_load(B.part + ((size_t)((unsigned)T & (PART_RING - 1)) * S + pk + in) * MSG_WORDS, pm2);
      intake_one(pk + in, pm2, T, SITE_HEAD_TAIL, &s_fail);
    }
    named_sync(BAR_END, nthr);
    if (s_fail) return;
    if (is_cs && tid < N) {
      const int j = tid;
      ExactBest eb;
      eb.init();
      for (int d = 0; d < hl; ++d) {
        const double e = hwr[((int)(t & (HWR - 1)) * L + d) * N + j] + m.survT[(size_t)j * D + d];
        // the tail reads delta[t-1-d] = delta[T-2-d]
        const int dr = (int)((T - 2 - d) % (L + 1));
        const double* row = dstar_h + dr * N;
        const double* trj = trh + (size_t)j * N;
        for (int i = 0; i < N; ++i) eb.offer((e + row[i]) + trj[i], d, i);
      }
      const int a = B.seg_first[j], b = a + B.seg_count[j];
      const int tb_ = (int)(T & 1) * S;  // the tail partials' buffer
      for (int k = a; k < b; ++k)
        if (pwd[tb_ + k] != EMPTY_D) eb.offer_key(pwk[tb_ + k], pwd[tb_ + k], pwi[tb_ + k]);
      if (eb.d == IDX_NONE) { eb.d = 0; eb.i = 0; }
      tail[j] = eb.value();
      B.psi[(size_t)t * N + j] = pack_psi(eb.d, eb.i);
    }
    named_sync(BAR_END, nthr);
  }

  // Backtrace (src/hsmm.cu:139-170).
  if (warp == 0) {
    int cur = 0;
    double best = tail[0];
    for (int n = 1; n < N; ++n)
      if (tail[n] > best) { best = tail[n]; cur = n; }
    long long t = T - 1;
    int bad = 0;
    while (t >= 0) {
      uint32_t wv = 0;
      if (lane == 0) wv = B.psi[(size_t)t * N + cur];
      wv = __shfl_sync(0xffffffffu, wv, 0);
      const long long len = (long long)(wv >> 16) + 1;
      const int prev = (int)(wv & 0xffffu);
      if (len > t + 1 || prev >= N) { bad = 1; break; }
      for (long long k = t - len + 1 + lane; k <= t; k += 32) B.path[k] = cur;
      t -= len;
      cur = prev;
    }
    if (lane == 0) {
      if (B.loglik) *B.loglik = best;
      if (bad) atomicCAS(B.status, 0, -8);
    }
  }
}

template <bool GW>
__global__ void __launch_bounds__(GRID_THREADS, 1) grid_decode_kernel(ModelView m, GridParams P, GridBufs B) {
  extern __shared__ __align__(16) unsigned char smem[];
  if (ld_relaxed_i32(B.abort_flag)) return;  // rejected observations
  if (blockIdx.x == 0) {
    grid_head(m, P, B, smem);
  } else if (threadIdx.x < (GW ? WORKER_THREADS_GW : WORKER_THREADS) + WORKER_SERVICE) {
    grid_worker<GW>(m, P, B, smem);
  }
}

}  // namespace tv
