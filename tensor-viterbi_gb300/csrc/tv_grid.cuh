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
constexpr int WORKER_THREADS = 256;     // a worker CTA keeps 8 warps (window in shared memory); the rest exit
constexpr int WORKER_THREADS_GW = 512;  // 16 warps when the window is in global memory (more loads in flight)
constexpr int GRID_L = 8;            // head candidates d < L (a power of two)
constexpr int CK_STRIDE = 32;      // checkpoint stride of the early window sums
constexpr int PART_RING = 32;      // steps of worker partials in flight
constexpr int SLOT_RING = 64;      // slot messages kept
constexpr int SLOT_WORDS = 5;      // ctil (2), dsel (2), itil (1)
constexpr int HEAD_GROUP = 4;      // lanes per state in the head's matvec (2 when N is too large for 4)
constexpr int GRID_MAX_N = 128;    // packed coarse scores keep the state index in 7 bits
constexpr int COARSE_F = 14;       // fraction bits of the packed coarse matvec scores
constexpr int COARSE_CLAMP = (1 << 23) - 1;
constexpr int EMPTY_D = 0xffff;
constexpr int TV_ETIMEOUT_DEV = -10;

struct GridParams {
  int G, L, S, Rd, M;
  long long chunk;  // largest worker range, in cells
  int max_seg;
  unsigned long long w_qd, w_dur, w_tr, w_ctil, w_dsel, w_acc0, w_acc1, w_itil, w_red, w_emw, w_bytes;
  int w_global;                  // the window lives in global memory (L2), not in shared memory
  unsigned long long w_gstride;  // bytes of one worker's window in global memory
  // head shared-memory offsets
  unsigned long long h_qcp, h_qtr, h_trh, h_dqcp, h_dq, h_ptil, h_base, h_dstar, h_ctil, h_itil, h_hwr, h_qd, h_dur,
      h_prek, h_pred, h_prei, h_prew, h_preq, h_pwq, h_pwk, h_pwd, h_pwi, h_psirec, h_tail, h_bytes;
  int trans_smem;     // the exact transition matrix is kept in the head's shared memory
  int qtr_smem;       // so is its fixed-point copy (else computed from the exact one)
  int cs_dense;       // critical threads of the dense (one lane per state) phase: N rounded up to 32
  int st_threads;     // state helper threads: N rounded up to 32
  int in_threads;     // intake threads: S rounded up to 32
  int block;          // threads per CTA: the head's roles (at least WORKER_THREADS)
  int head_group;     // matvec lanes per state in the head (4, or 2 for large N)
  int qf;             // fraction bits of the fixed-point scores
  int Np;             // N rounded up to 16 (packed coarse matvec rows)
  int cs_threads;     // critical-section threads (4 lanes per state, whole warps)
  int coarse_shift;   // fine-to-coarse right shift (f - COARSE_F)
  int coarse_margin;  // certified coarse i-margin, coarse units
  long long timeout;
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
       SITE_HEAD_TAIL = 5 };

__device__ __forceinline__ void grid_fail(const GridBufs& B, int code, int site) {
  if (atomicCAS(B.status, 0, code) == 0) *B.site = site;
  atomicExch(B.abort_flag, 1);
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

// Named barrier of the worker threads only (the rest of the CTA has exited).
// The non-aligned barrier counts threads, so lanes of a warp may arrive apart
// (after a lane-0 wait, say); the aligned bar.sync would need the warp
// converged, which the compiler does not ensure before inline assembly.
template <int WT>
__device__ __forceinline__ void worker_sync() {
  asm volatile("barrier.sync 1, %0;" ::"r"(WT) : "memory");
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
  TaggedMsg msg;
  const bool empty = eb.d == IDX_NONE;
  msg_pack(msg, tag, eb.value(), empty ? EMPTY_D : eb.d, empty ? 0 : eb.i);
  msg_store(B.part + ((size_t)ring * P.S + seg) * MSG_WORDS, msg);
}

// ---------------------------------------------------------------------------
// Worker CTA (WORKER_THREADS threads, WORKER_THREADS_GW with the window in global memory)
// ---------------------------------------------------------------------------
// GW: the worker's window (slot scores, selected deltas, window sums, argmax
// words) lives in a private global-memory buffer, served by L1/L2, and the
// duration and transition rows are read from the model's tables; used when
// N*D is too large for the workers' shared memory.
template <bool GW>
__device__ void grid_worker(const ModelView& m, const GridParams& P, const GridBufs& B, unsigned char* sm) {
  constexpr int L = GRID_L;
  constexpr int WT = GW ? WORKER_THREADS_GW : WORKER_THREADS;
  constexpr int NW = WT / 32;
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
  const long long* qd = GW ? m.qdurT + (size_t)ja * D : qd_s;
  const double* dur = GW ? m.durT + (size_t)ja * D : dur_s;
  const double* tr = GW ? m.trans + (size_t)ja * N : tr_s;
  long long* ctil = (long long*)(wb + P.w_ctil);      // [ncell]
  double* dsel = (double*)(wb + P.w_dsel);            // [ncell]
  double* acc_cur = (double*)(wb + P.w_acc0);         // [ncell] E_t
  double* acc_nxt = (double*)(wb + P.w_acc1);         // [ncell] E_{t+1}
  unsigned short* itil = (unsigned short*)(wb + P.w_itil);
  Top2* red = (Top2*)(sm + P.w_red);                  // [nseg][NW]
  ExactBest* ered = (ExactBest*)(sm + P.w_red);
  double* emw = (double*)(sm + P.w_emw);              // [2][max_seg] emission of the fold's step
  __shared__ int s_bad;

  if (!GW) {
    for (long long k = tid; k < (long long)nseg * D; k += WT) {
      qd_s[k] = m.qdurT[(size_t)ja * D + k];
      dur_s[k] = m.durT[(size_t)ja * D + k];
    }
    for (int k = tid; k < nseg * N; k += WT) tr_s[k] = m.trans[(size_t)ja * N + k];
  }
  if (tid == 0) s_bad = 0;
  worker_sync<WT>();

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
  worker_sync<WT>();

  int r0 = 0;  // (t-1) % D
  for (long long t = 1; t < T; ++t) {
    const int tau = (int)(t < D ? t : D);
    const unsigned prow = (unsigned)t & (PART_RING - 1);
    const long long t1 = t + 1;
    int r0n = r0 + 1;  // t % D: the slot that enters at step t+1 (d = 0 then)
    if (r0n == D) r0n = 0;
    if (tid < nseg) {
      if (t + 2 < T) emw[(int)((t + 2) & 1) * P.max_seg + tid] = em_pf;
      if (t + 3 < T) em_pf = m.em[(size_t)ob_pf * N + ja + tid];
      if (t + 4 < T) ob_pf = B.obs[t + 4];
    }

    // Phase 1: fixed-point scan over d in [L, tau), fused with the exact
    // window folds of step t+1 into the other buffer (src/hsmm.cu:298-310):
    // E_{t+1}[d] = E_t[d-1] + em_{t+1}, E_{t+1}[0] = 0 + em_{t+1}.  The FP64
    // adds overlap the integer scan.
    const bool fold = (t1 < T) && (t1 > D + 1);
    for (int s = 0; s < nseg; ++s) {
      int rb, re;
      seg_of(s, rb, re);
      const long long* ct = ctil + s * D - off0;
      const long long* q = qd + s * D;
      const double* ac = acc_cur + s * D - off0;
      double* an = acc_nxt + s * D - off0;
      const double em1 = fold ? emw[(int)(t1 & 1) * P.max_seg + s] : 0.0;
      Top2 tb;
      tb.init();
#pragma unroll 4
      for (int r = rb + tid; r < re; r += WT) {
        int d = r0 - r;
        if (d < 0) d += D;
        if (d >= L && d < tau) tb.push(ct[r] + q[d], d);
        if (fold) an[r] = ((r == r0n) ? 0.0 : ac[r]) + em1;
      }
      tb.warp_reduce();
      if (lane == 0) red[s * NW + warp] = tb;
    }
    worker_sync<WT>();

    // Phase 2a: certified exact winner per segment (warps take segments in
    // turn), sent to the head.
    for (int s = warp; s < nseg; s += NW) {
      const int j = ja + s;
      int rb, re;
      seg_of(s, rb, re);
      Top2 tb;
      tb.init();
      if (lane < NW) tb = red[s * NW + lane];
      tb.warp_reduce();
      ExactBest eb;
      eb.init();
      if (tb.x1 != IDX_NONE) {
        const int d1 = tb.x1;
        int r1 = r0 - d1;
        if (r1 < 0) r1 += D;
        const int c1 = s * D + r1 - off0;
        const unsigned short it = itil[c1];
        const bool amb = (it & 0x8000) || ((tb.b1 - tb.b2) <= m.margin);
        if (!amb) {
          if (lane == 0) {
            const int i1 = it & 0x7fff;
            const double e = (t > D) ? acc_cur[c1] : early_window(m, B.ck, P.M, B.obs, t, d1, j);
            eb.set((e + dsel[c1]) + (tr[s * N + i1] + dur[s * D + d1]), d1, i1);
          }
        } else {
          // Re-score every candidate inside the margin exactly.
          const long long thr = tb.b1 - m.margin;
          bool ok = true;
          for (int r = rb + lane; r < re; r += 32) {
            int d = r0 - r;
            if (d < 0) d += D;
            if (d < L || d >= tau) continue;
            const int c = s * D + r - off0;
            if (ctil[c] + qd[s * D + d] < thr) continue;
            const double e = (t > D) ? acc_cur[c] : early_window(m, B.ck, P.M, B.obs, t, d, j);
            const double du = dur[s * D + d];
            for (int i = 0; i < N && ok; ++i) {
              double dv;
              ok = load_dstar(B, P, N, t - 1 - d, i, dv);
              if (ok) eb.offer((e + dv) + (tr[s * N + i] + du), d, i);
            }
          }
          eb.warp_reduce();
          if (!__all_sync(0xffffffffu, ok)) {
            if (lane == 0) { grid_fail(B, TV_ETIMEOUT_DEV, SITE_WORKER_RESCORE); s_bad = 1; }
          }
        }
      }
      if (lane == 0) send_partial(B, P, (unsigned)t, prow, seg0 + s, eb);
    }
    // Phase 2b: intake of the slot that enters the worker domain at step t+1
    // (s' = t-L, d = L then); the last warp, one lane per segment.  Lane 0
    // waits for the slot message even when the slot is not its own: that is
    // the flow control that keeps a worker at most L steps ahead of the head
    // (its partials ring holds PART_RING steps).
    if (warp == NW - 1 && lane < nseg && t + 1 < T && t - L >= 0) {
      const long long sp = t - L;
      int rn = r0 + 1 - L;
      if (rn < 0) rn += D;
      int rb, re;
      seg_of(lane, rb, re);
      const unsigned tag = (unsigned)(sp + 1);
      const unsigned long long* msg =
          B.slot_msg + ((size_t)((unsigned)sp & (SLOT_RING - 1)) * N + ja + lane) * SLOT_WORDS;
      unsigned long long cbits, dbits, ibits;
      if (rn < rb || rn >= re) {
        if (lane == 0 && !tagged64_load(msg, tag, cbits, B.abort_flag, P.timeout)) {
          grid_fail(B, TV_ETIMEOUT_DEV, SITE_WORKER_SLOT);
          s_bad = 1;
        }
      } else {
        bool ok = tagged64_load(msg, tag, cbits, B.abort_flag, P.timeout) &&
                  tagged64_load(msg + 2, tag, dbits, B.abort_flag, P.timeout);
        if (ok) {
          unsigned long long iw = ld_relaxed_u64(msg + 4);
          const long long t0 = clock64();
          while ((unsigned)(iw >> 32) != tag) {
            if (ld_relaxed_i32(B.abort_flag) || clock64() - t0 > P.timeout) { ok = false; break; }
            iw = ld_relaxed_u64(msg + 4);
          }
          ibits = iw;
        }
        if (ok) {
          const int c = lane * D + rn - off0;
          ctil[c] = (long long)cbits;
          dsel[c] = __longlong_as_double((long long)dbits);
          itil[c] = (unsigned short)(ibits & 0xffff);
        } else {
          grid_fail(B, TV_ETIMEOUT_DEV, SITE_WORKER_SLOT);
          s_bad = 1;
        }
      }
    }
    // Phase 2c: at t+1 = D+1 the first fold starts from the reference's
    // newest-first sums of step D: E_{D+1}[d] = E_D[d-1] + em_{D+1}.
    const bool seed = (t1 < T) && (t1 == D + 1);
    if (seed) {
      const int ot1 = B.obs[t1];
      for (int s = 0; s < nseg; ++s) {
        int rb, re;
        seg_of(s, rb, re);
        const int j = ja + s;
        const double em1 = m.em[(size_t)ot1 * N + j];
        double* an = acc_nxt + s * D - off0;
        for (int r = rb + tid; r < re; r += WT) {
          int d = r0n - r;
          if (d < 0) d += D;
          const double base = (d == 0) ? 0.0 : early_window(m, B.ck, P.M, B.obs, D, d - 1, j);
          an[r] = base + em1;
        }
      }
    }
    worker_sync<WT>();
    if (s_bad) return;
    if (fold || seed) {
      double* x = acc_cur;
      acc_cur = acc_nxt;
      acc_nxt = x;
    }
    r0 = r0n;
  }

  // Tail at t = T-1: exhaustive exact scan of the worker's cells with the
  // survival function (src/hsmm.cu:101-137), one partial per segment.
  {
    const long long t = T - 1;
    const int tau = (int)(t < D ? t : D);
    const int rt = t >= 1 ? (int)((t - 1) % D) : 0;
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
        const double E = (t > D) ? acc_cur[c] : early_window(m, B.ck, P.M, B.obs, t, d, j);
        const double e = E + m.survT[(size_t)j * D + d];
        for (int i = 0; i < N && ok; ++i) {
          double dv;
          ok = load_dstar(B, P, N, t - 1 - d, i, dv);
          if (ok) eb.offer((e + dv) + tr[s * N + i], d, i);
        }
      }
      if (!ok) {
        grid_fail(B, TV_ETIMEOUT_DEV, SITE_WORKER_TAIL);
        s_bad = 1;
      }
      eb = worker_reduce_exact<WT>(eb, ered);
      if (s_bad) return;
      if (tid == 0) send_partial(B, P, (unsigned)T, (unsigned)T & (PART_RING - 1), seg0 + s, eb);
    }
  }
}

// ---------------------------------------------------------------------------
// Head CTA
//
// The serial critical path of a step is: delta[t-1] final -> B[t-1][j] =
// max_i(trans[j][i] + delta[t-1][i]) for every j -> the d = 0 candidate ->
// merge -> delta[t].  Only that chain runs in the critical warps:
//   * the matvec, 4 lanes per state, in packed int32: coarse score << 7 |
//     (127 - i), so one integer max yields the value and the lowest index;
//     its runner-up gap is certified against a coarse margin, else a fine
//     int64 pass decides;
//   * then one lane per state (the dense phase): the d = 0 candidate's
//     fixed-point score W0 against Wtop, the best fixed-point score over
//     d >= 1 that the helpers prepared one step ahead with the exact winner
//     among d >= 1.  When W0 trails Wtop by more than the certified margin,
//     delta[t] is that winner and no floating-point operation runs; otherwise
//     the d = 0 score is computed exactly (two dependent FP64 adds) and
//     compared.
// FP64 instructions cost the same pipe time whatever the number of active
// lanes, so exact scores are computed one lane per state, never one lane in
// four.
// The helper warps (the rest of the CTA) prepare step t+1 meanwhile: intake
// of the workers' partial winners (loaded a step ahead), window sums (copied
// asynchronously three steps ahead from a table built before the launch),
// the candidates d = 1..L-1 in fixed point, certification, and in a dense
// phase the exact score of the winner when it is one of them; also all global
// stores.  A named barrier hands the matvec result (slot t-1) from the
// critical warps to the helpers inside the step.
// ---------------------------------------------------------------------------
constexpr int HWR = 4;  // rows of window sums kept by the head: steps t .. t+3

// Named barriers of the head CTA (the CTA-wide barrier 0 is used only while
// every thread is alive; threads without a role leave before the steps).
// Non-aligned forms: they count threads, so a warp whose lanes took different
// branches may arrive lane by lane.
enum { BAR_STEP = 1, BAR_SLOT = 2, BAR_DENSE = 3, BAR_PW = 4 };
__device__ __forceinline__ void named_sync(int id, int count) {
  asm volatile("barrier.sync %0, %1;" ::"r"(id), "r"(count) : "memory");
}
__device__ __forceinline__ void named_arrive(int id, int count) {
  asm volatile("barrier.arrive %0, %1;" ::"r"(id), "r"(count) : "memory");
}

__device__ __forceinline__ void cp_async16(void* smem_dst, const void* gmem_src) {
  const unsigned d = (unsigned)__cvta_generic_to_shared(smem_dst);
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(d), "l"(gmem_src) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
__device__ __forceinline__ void cp_async_wait_all_but_1() { asm volatile("cp.async.wait_group 1;" ::: "memory"); }

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

template <int G4>
__device__ __forceinline__ void group_reduce_exact(ExactBest& eb, unsigned gmask) {
#pragma unroll
  for (int o = G4 / 2; o > 0; o >>= 1) {
    const long long ok = __shfl_xor_sync(gmask, eb.k, o);
    const int od = __shfl_xor_sync(gmask, eb.d, o);
    const int oi = __shfl_xor_sync(gmask, eb.i, o);
    eb.offer_key(ok, od, oi);
  }
}

// A worker segment's exact winner, kept as its order key and its fixed-point
// value (the value of the segment's best candidate, to within half a unit).
__device__ __forceinline__ void take_partial(const TaggedMsg& pm, int k, int qf, long long* pwq, long long* pwk,
                                             int* pwd, int* pwi) {
  double v;
  int d, i;
  msg_unpack(pm, v, d, i);
  pwq[k] = d != EMPTY_D ? fixed_from_double(v, qf) : 0;
  pwk[k] = order_key(v);
  pwd[k] = d;
  pwi[k] = i;
}

template <int G4>
__device__ void grid_head(const ModelView& m, const GridParams& P, const GridBufs& B, unsigned char* sm) {
  constexpr int L = GRID_L;
  const int N = m.N, D = m.D, S = P.S, Np = P.Np;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const unsigned gmask = ((1u << G4) - 1) << ((lane / G4) * G4);
  const long long T = B.T;
  const long long margin = m.margin;
  int* Qcp = (int*)(sm + P.h_qcp);                    // [N][Np] packed coarse trans
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
  long long* qd_h = (long long*)(sm + P.h_qd);        // [N][L]
  double* dur_h = (double*)(sm + P.h_dur);            // [N][L]
  long long* prek = (long long*)(sm + P.h_prek);      // [2][N] exact winner over d >= 1: order key
  int* pred = (int*)(sm + P.h_pred);
  int* prei = (int*)(sm + P.h_prei);
  long long* prew = (long long*)(sm + P.h_prew);      // [2][N] best fixed-point score over d >= 1
  long long* preq = (long long*)(sm + P.h_preq);      // [2][N] fixed-point value of the exact winner
  long long* pwq = (long long*)(sm + P.h_pwq);        // [S] worker partials of the next step
  long long* pwk = (long long*)(sm + P.h_pwk);
  int* pwd = (int*)(sm + P.h_pwd);
  int* pwi = (int*)(sm + P.h_pwi);
  uint32_t* psirec = (uint32_t*)(sm + P.h_psirec);    // [2][N] back-pointer word of a step
  double* tail = (double*)(sm + P.h_tail);
  __shared__ int s_fail;
  const int sh = P.coarse_shift;
  // Roles, by thread range:
  //   [0, cs)             critical: the matvec, 4 lanes per state; the first
  //                       cs_dense threads then run the dense phase, one lane per state
  //   [cs, cs+st)         state helpers, one lane per state: step t+1's
  //                       candidates, certification and exact winner, stores
  //   [cs+st, cs+st+in)   intake of the workers' partial winners, one lane per
  //                       segment; the first of these warps also computes the coarse base
  // Threads beyond these leave once the tables are set up.
  const int cs = P.cs_threads, st = P.st_threads, in = P.in_threads;
  const int nthr = cs + st + in;
  const bool is_cs = tid < cs;
  const bool is_st = !is_cs && tid < cs + st;
  const bool is_in = !is_cs && !is_st && tid < nthr;
  const int gj = tid / G4, gl = tid % G4;              // critical: state and lane of this group
  const int sj = tid - cs;                             // state helper: state
  const int pk = tid - cs - st;                        // intake: segment
  const bool has_sj = is_st && sj < N;
  const bool has_pk = is_in && pk < S;
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
      Qcp[k] = c * 128 + (127 - i);
    } else {
      Qcp[k] = INT_MIN;
    }
  }
  for (int k = tid; k < N * N; k += blockDim.x) {
    if (P.qtr_smem) qtr_s[k] = m.qtr[k];
    if (P.trans_smem) trh_s[k] = m.trans[k];
  }
  for (int k = tid; k < N * L; k += blockDim.x) {
    const int jj = k / L, d = k % L;
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
  if (tid == 0) s_fail = 0;
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
  // worker partials of step 1 (all empty: no d >= L yet), and the prefetch of step 2
  TaggedMsg pm;
  if (has_pk && T > 1) {
    const unsigned long long* src = B.part + ((size_t)(1 & (PART_RING - 1)) * S + pk) * MSG_WORDS;
    msg_load(src, pm);
    if (!msg_wait(src, 1u, pm, B.abort_flag, P.timeout)) {
      grid_fail(B, TV_ETIMEOUT_DEV, SITE_HEAD_PARTIAL);
      s_fail = 1;
    } else {
      take_partial(pm, pk, P.qf, pwq, pwk, pwd, pwi);
    }
    if (T > 2) msg_load(B.part + ((size_t)(2 & (PART_RING - 1)) * S + pk) * MSG_WORDS, pm);
  }
  __syncthreads();
  if (s_fail) return;
  for (int jj = tid; jj < N; jj += blockDim.x) {
    const int a = B.seg_first[jj], b = a + B.seg_count[jj];
    const long long p1 = ptil[N + jj];
    long long W = QNEG;
    for (int k = a; k < b; ++k)
      if (pwd[k] != EMPTY_D) W = max(W, pwq[k] - p1);
    ExactBest eb;
    eb.init();
    for (int k = a; k < b; ++k)
      if (pwd[k] != EMPTY_D && pwq[k] - p1 >= W - margin) eb.offer_key(pwk[k], pwd[k], pwi[k]);
    prew[(1 & 1) * N + jj] = W;
    prek[(1 & 1) * N + jj] = eb.k;
    pred[(1 & 1) * N + jj] = eb.d;
    prei[(1 & 1) * N + jj] = eb.i;
    preq[(1 & 1) * N + jj] = eb.d != IDX_NONE ? fixed_from_double(eb.value(), P.qf) : 0;
  }
  __syncthreads();
  if (tid >= nthr) return;  // no role in the steps

  // Register pipelines: a state helper keeps the prefix term of step t+2 and
  // the observation of step t+3; an intake lane the partial message of step
  // t+2 (in pm); a dense critical lane the initialisation score of step t+1.
  long long qe_pf = 0;
  int ob_q = 0;
  if (has_sj) {
    if (2 < T) qe_pf = m.qem[(size_t)B.obs[2] * N + sj];
    if (3 < T) ob_q = B.obs[3];
  }
  double di_cur = 0.0;  // initialisation score of step t, state tid (dense critical lanes)
  if (tid < N && 1 < D) di_cur = __ldcg(B.dinit + (size_t)1 * N + tid);
  const int hw_chunks = L * N / 2;  // 16-byte pieces of a window-sum row

  int drow_prev = 0;  // (t-1) % (L+1): row of delta[t-1] in dstar_h
  int rdrow = 1;      // t % Rd: row of delta[t] in the tagged ring
  for (long long t = 1; t < T; ++t) {
    const int cur = (int)(t & 1), prv = cur ^ 1;
    const int drow = drow_prev + 1 == L + 1 ? 0 : drow_prev + 1;  // t % (L+1)
    const int hrow = (int)((t - 1) & (L - 1));                      // slot t-1 in ctil_h
    const long long t1 = t + 1;
    const bool next = t1 < T;
    const int nxt = cur ^ 1;  // (t+1) & 1
    if (is_cs) {
      // ================= critical warps =================
      double di_next = 0.0;
      if (tid < N && t + 1 < D) di_next = __ldcg(B.dinit + (size_t)(t + 1) * N + tid);
      if (gj < N) {
        const int j = gj;
        // packed coarse matvec over i for slot t-1
        int b1 = INT_MIN, b2 = INT_MIN;
        const int* qrow = Qcp + j * Np;
        const int* dv = dqcp + prv * Np;
        for (int i4 = gl * 4; i4 < Np; i4 += 4 * G4) {
          const int4 a = *reinterpret_cast<const int4*>(qrow + i4);
          const int4 b = *reinterpret_cast<const int4*>(dv + i4);
          packed_push(a.x + b.x, b1, b2);
          packed_push(a.y + b.y, b1, b2);
          packed_push(a.z + b.z, b1, b2);
          packed_push(a.w + b.w, b1, b2);
        }
#pragma unroll
        for (int o = G4 / 2; o > 0; o >>= 1) {
          const int o1 = __shfl_xor_sync(gmask, b1, o);
          const int o2 = __shfl_xor_sync(gmask, b2, o);
          const int lo = min(b1, o1);
          b1 = max(b1, o1);
          b2 = max(max(b2, o2), lo);
        }
        int ifine = 127 - (b1 & 127);
        bool amb = ((b1 >> 7) - (b2 >> 7)) <= P.coarse_margin;
        long long bfine;
        if (!amb) {
          bfine = qtr_at(j, ifine) + dq[prv * N + ifine];
        } else {
          // fine int64 pass decides (and certifies with the fine margin)
          Top2 tb;
          tb.init();
          // (a whole row: the shared copy, else the global one, whose loads
          // are independent and overlap, unlike N dependent conversions)
          const long long* qrow_f = P.qtr_smem ? qtr_s + (size_t)j * N : m.qtr + (size_t)j * N;
          for (int i = gl; i < N; i += G4) tb.push(qrow_f[i] + dq[prv * N + i], i);
#pragma unroll
          for (int o = G4 / 2; o > 0; o >>= 1) {
            const long long ob1 = __shfl_xor_sync(gmask, tb.b1, o);
            const long long ob2 = __shfl_xor_sync(gmask, tb.b2, o);
            const int ox1 = __shfl_xor_sync(gmask, tb.x1, o);
            tb.merge(ob1, ox1, ob2);
          }
          ifine = tb.x1;
          bfine = tb.b1;
          amb = (tb.b1 - tb.b2) <= margin;
        }
        if (gl == 0) {
          ctil_h[hrow * N + j] = bfine - ptil[(int)((t - 1) & 3) * N + j];
          itil_h[hrow * N + j] = (unsigned short)(ifine | (amb ? 0x8000 : 0));
        }
      }
      named_arrive(BAR_SLOT, cs + st);  // slot t-1 ready for the state helpers
      if (tid < P.cs_dense) {
        named_sync(BAR_DENSE, cs);
        if (tid < N) {
          // dense phase, one lane per state; the exact d = 0 score of the
          // certified argmax over i is computed before it is known to be needed
          const int dj = tid;
          const long long W0 = ctil_h[hrow * N + dj] + qd_h[dj * L];  // the d = 0 candidate, fixed point
          const unsigned short it = itil_h[hrow * N + dj];
          const long long Wt = prew[cur * N + dj];
          const long long pk0 = prek[cur * N + dj];
          const int pd0 = pred[cur * N + dj], pi0 = prei[cur * N + dj];
          const long long pq0 = preq[cur * N + dj];
          const int i1 = it & 0x7fff;
          const double e0 = hwr[(int)(t & (HWR - 1)) * L * N + dj];
          const double du0 = dur_h[dj * L];
          // src/hsmm.cu:341-346 with E_t[0]
          const double V0 = (e0 + dstar_h[drow_prev * N + i1]) + (trh[(size_t)dj * N + i1] + du0);
          const long long q0 = quantize(V0, m.scale);
          long long kk = pk0, fq = pq0;
          int dd = pd0, ii = pi0;
          if (W0 >= Wt - margin) {
            ExactBest eb;
            if (!(it & 0x8000)) {
              eb.set(V0, 0, i1);
            } else {
              eb.init();
              const double* row = dstar_h + drow_prev * N;
              const double* trj = trh + (size_t)dj * N;
              for (int i = 0; i < N; ++i) eb.offer((e0 + row[i]) + (trj[i] + du0), 0, i);
            }
            if (W0 <= Wt + margin) eb.offer_key(pk0, pd0, pi0);
            kk = eb.k;
            dd = eb.d;
            ii = eb.i;
            if (dd == 0) fq = (it & 0x8000) ? quantize(eb.value(), m.scale) : q0;
          }
          double fin = key_value(kk);
          uint32_t wv = pack_psi(dd, ii);
          // t < D: the induction result replaces the initialisation score only
          // when strictly larger (src/hsmm.cu:353-358).
          if (t < D && !(kk > order_key(di_cur))) {
            fin = di_cur;
            wv = pack_psi((int)t, 0);
            fq = quantize(fin, m.scale);
          }
          dstar_h[drow * N + dj] = fin;
          dq[cur * N + dj] = fq;
          dqcp[cur * Np + dj] = coarse_of(fq - basebuf[cur], sh) * 128;
          psirec[cur * N + dj] = wv;
        }
      } else {
        named_arrive(BAR_DENSE, cs);
      }
      di_cur = di_next;
    } else if (is_st) {
      // ============ state helpers: prepare step t+1, one lane per state ============
      // window sums of step t+3 into the ring; the copies of step t+2 are
      // complete before this step's closing barrier
      for (int c = sj; c < hw_chunks; c += st)
        if (t + 3 < T)
          cp_async16(hwr + (int)((t + 3) & (HWR - 1)) * L * N + c * 2, B.hwin + (size_t)(t + 3) * L * N + c * 2);
      cp_async_commit();
      cp_async_wait_all_but_1();
      if (has_sj) {
        if (next) {
          ptil[(int)(t1 & 3) * N + sj] = ptil[(int)(t & 3) * N + sj] + qe_pf;  // P(t+1)
          if (t + 2 < T) qe_pf = m.qem[(size_t)ob_q * N + sj];
          if (t + 3 < T) ob_q = B.obs[t + 3];
        }
        // results of step t-1 to global memory
        if (t >= 2) {
          B.psi[(size_t)(t - 1) * N + sj] = psirec[prv * N + sj];
          tagged64_store(B.dstar + ((size_t)(rdrow == 0 ? P.Rd - 1 : rdrow - 1) * N + sj) * 2, (unsigned)t,
                         (unsigned long long)__double_as_longlong(dstar_h[drow_prev * N + sj]));
        }
      }
      named_sync(BAR_SLOT, cs + st);  // the critical warps published slot t-1
      if (has_sj) {
        // slot t-1 message for the workers
        unsigned long long* msg =
            B.slot_msg + ((size_t)((unsigned)(t - 1) & (SLOT_RING - 1)) * N + sj) * SLOT_WORDS;
        const unsigned tag = (unsigned)t;
        const unsigned short itv = itil_h[hrow * N + sj];
        tagged64_store(msg, tag, (unsigned long long)ctil_h[hrow * N + sj]);
        tagged64_store(msg + 2, tag,
                       (unsigned long long)__double_as_longlong(dstar_h[drow_prev * N + (itv & 0x7fff)]));
        st_relaxed_u64(msg + 4, ((unsigned long long)tag << 32) | itv);
      }
      named_sync(BAR_PW, st + in);  // the intake lanes took in the partials of step t+1
      if (has_sj && next) {
        // Every candidate d >= 1 of step t+1 in fixed point: d = 1..L-1 here
        // (slots t-d), d >= L as the workers' winners, whose fixed-point
        // scores are their values minus the prefix P(t+1).  Written for
        // instruction-level parallelism: one lane carries a state, so its
        // loads are issued together and the exact score of the best short
        // candidate is computed before it is known to be needed.
        const int tau1 = (int)(t1 < D ? t1 : D);
        const int hl1 = tau1 < L ? tau1 : L;
        const long long p1 = ptil[(int)(t1 & 3) * N + sj];
        long long Wd[L];
        unsigned short itd[L];
#pragma unroll
        for (int d = 1; d < L; ++d) {
          const int row = (int)((t - d) & (L - 1));
          Wd[d] = d < hl1 ? ctil_h[row * N + sj] + qd_h[sj * L + d] : QNEG;
          itd[d] = itil_h[row * N + sj];
        }
        long long Wh = QNEG;
        int dh = 0, ih = 0, hamb = 0;
#pragma unroll
        for (int d = 1; d < L; ++d)
          if (Wd[d] > Wh) {
            Wh = Wd[d];
            dh = d;
            ih = itd[d] & 0x7fff;
            hamb = itd[d] & 0x8000;
          }
        double Vh = 0.0;
        long long qh = 0;
        if (dh > 0) {
          int dr = drow_prev + 1 - dh;  // row of delta[t-dh]
          if (dr < 0) dr += L + 1;
          const double e = hwr[((int)(t1 & (HWR - 1)) * L + dh) * N + sj];
          Vh = (e + dstar_h[dr * N + ih]) + (trh[(size_t)sj * N + ih] + dur_h[sj * L + dh]);
          qh = quantize(Vh, m.scale);
        }
        long long Wl = Wh;
        for (int k = k0; k < k1; ++k)
          if (pwd[k] != EMPTY_D) Wl = max(Wl, pwq[k] - p1);
        const long long thr = Wl - margin;
        // exact winner among the candidates within the margin of the best,
        // with its fixed-point value
        ExactBest eb;
        eb.init();
        long long qb = 0;
        for (int k = k0; k < k1; ++k)
          if (pwd[k] != EMPTY_D && pwq[k] - p1 >= thr && eb.better_key(pwk[k], pwd[k], pwi[k])) {
            eb.k = pwk[k];
            eb.d = pwd[k];
            eb.i = pwi[k];
            qb = pwq[k];
          }
        int nh = 0;
#pragma unroll
        for (int d = 1; d < L; ++d) nh += Wd[d] >= thr ? 1 : 0;
        if (nh == 1 && !hamb) {
          const long long kh = order_key(Vh);
          if (eb.better_key(kh, dh, ih)) {
            eb.k = kh;
            eb.d = dh;
            eb.i = ih;
            qb = qh;
          }
        } else if (nh > 0) {
          // several short candidates in the margin, or an ambiguous argmax over i
          for (int d = 1; d < hl1; ++d) {
            if (Wd[d] < thr) continue;
            const double e = hwr[((int)(t1 & (HWR - 1)) * L + d) * N + sj];
            const double du = dur_h[sj * L + d];
            int dr = drow_prev + 1 - d;  // row of delta[t-d]
            if (dr < 0) dr += L + 1;
            const double* drw = dstar_h + dr * N;
            const double* trj = trh + (size_t)sj * N;
            const unsigned short it = itd[d];
            if (!(it & 0x8000)) {
              const int i1 = it & 0x7fff;
              eb.offer((e + drw[i1]) + (trj[i1] + du), d, i1);
            } else {
              for (int i = 0; i < N; ++i) eb.offer((e + drw[i]) + (trj[i] + du), d, i);
            }
          }
          qb = eb.d == IDX_NONE ? 0 : quantize(eb.value(), m.scale);
        }
        prew[nxt * N + sj] = Wl;
        prek[nxt * N + sj] = eb.k;
        pred[nxt * N + sj] = eb.d;
        prei[nxt * N + sj] = eb.i;
        preq[nxt * N + sj] = qb;
      }
    } else {
      // ============ intake: worker partials of step t+1, loaded during the previous step ============
      if (has_pk && next) {
        if (!msg_wait(B.part + ((size_t)((unsigned)t1 & (PART_RING - 1)) * S + pk) * MSG_WORDS, (unsigned)t1, pm,
                      B.abort_flag, P.timeout)) {
          grid_fail(B, TV_ETIMEOUT_DEV, SITE_HEAD_PARTIAL);
          s_fail = 1;
        } else {
          take_partial(pm, pk, P.qf, pwq, pwk, pwd, pwi);
        }
        if (t1 + 1 < T) msg_load(B.part + ((size_t)((unsigned)(t1 + 1) & (PART_RING - 1)) * S + pk) * MSG_WORDS, pm);
      }
      named_arrive(BAR_PW, st + in);
      // coarse base of step t+1: max_i delta[t-1] (the first intake warp)
      if (pk < 32) {
        long long mx = LLONG_MIN;
        for (int i = pk; i < N; i += 32) mx = max(mx, dq[prv * N + i]);
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) mx = max(mx, __shfl_xor_sync(0xffffffffu, mx, o));
        if (pk == 0) basebuf[nxt] = mx;
      }
    }
    drow_prev = drow;
    rdrow = rdrow + 1 == P.Rd ? 0 : rdrow + 1;
    named_sync(BAR_STEP, nthr);
    if (s_fail) return;
  }

  // Tail at t = T-1 (src/hsmm.cu:101-137).
  {
    const long long t = T - 1;
    const int tau = (int)(t < D ? t : D);
    const int hl = tau < L ? tau : L;
    if (has_pk) {
      const unsigned long long* src = B.part + ((size_t)((unsigned)T & (PART_RING - 1)) * S + pk) * MSG_WORDS;
      msg_load(src, pm);
      if (!msg_wait(src, (unsigned)T, pm, B.abort_flag, P.timeout)) {
        grid_fail(B, TV_ETIMEOUT_DEV, SITE_HEAD_TAIL);
        s_fail = 1;
      } else {
        take_partial(pm, pk, P.qf, pwq, pwk, pwd, pwi);
      }
    }
    named_sync(BAR_STEP, nthr);
    if (s_fail) return;
    if (is_cs && gj < N) {
      const int j = gj;
      ExactBest eb;
      eb.init();
      for (int d = gl; d < hl; d += G4) {
        const double e = hwr[((int)(t & (HWR - 1)) * L + d) * N + j] + m.survT[(size_t)j * D + d];
        // after the loop drow_prev is the row of delta[T-1]; the tail reads
        // delta[t-1-d] = delta[T-2-d]
        int dr = drow_prev - 1 - d;
        while (dr < 0) dr += L + 1;
        const double* row = dstar_h + dr * N;
        const double* trj = trh + (size_t)j * N;
        for (int i = 0; i < N; ++i) eb.offer((e + row[i]) + trj[i], d, i);
      }
      group_reduce_exact<G4>(eb, gmask);
      if (gl == 0) {
        const int a = B.seg_first[j], b = a + B.seg_count[j];
        for (int k = a; k < b; ++k)
          if (pwd[k] != EMPTY_D) eb.offer_key(pwk[k], pwd[k], pwi[k]);
        if (eb.d == IDX_NONE) { eb.d = 0; eb.i = 0; }
        tail[j] = eb.value();
        B.psi[(size_t)t * N + j] = pack_psi(eb.d, eb.i);
      }
    }
    named_sync(BAR_STEP, nthr);
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

template <bool GW, int G4>
__global__ void __launch_bounds__(GRID_THREADS, 1) grid_decode_kernel(ModelView m, GridParams P, GridBufs B) {
  extern __shared__ __align__(16) unsigned char smem[];
  if (ld_relaxed_i32(B.abort_flag)) return;  // rejected observations
  if (blockIdx.x == 0) {
    grid_head<G4>(m, P, B, smem);
  } else if (threadIdx.x < (GW ? WORKER_THREADS_GW : WORKER_THREADS)) {
    grid_worker<GW>(m, P, B, smem);
  }
}

}  // namespace tv
