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
//           max-plus matvec for the newest slot s = t-1 (published to the
//           workers), the candidates d < L, the merge with the workers'
//           exact partial winners, the initialisation rule for t < D, the
//           exact delta[t] and the back-pointers.
//   workers for their cells: the exact window fold (t > D), the fixed-point
//           scan over d >= L, the certified exact local winner, published
//           as a tagged message.  A worker needs slot t-1-L to run step t,
//           so it may run up to L steps ahead of the head; the cross-SM
//           latency is overlapped instead of paid every step.
// After step T-1 the tail (survival in place of the duration pmf) is one
// more round of the same protocol with an exhaustive exact scan, and the head
// backtraces.
//
// While t <= D the reference rebuilds the window sums newest-first
// (src/hsmm.cu:311-322); a worker then takes the exact value of its winner
// from a checkpoint table g_t(k*K) built before the launch plus at most K-1
// additions.
#pragma once
#include "tv_cta.cuh"
#include "tv_device.cuh"
#include "tv_sync.cuh"

namespace tv {

constexpr int GRID_THREADS = 1024;
constexpr int GRID_L = 4;          // head candidates d < L
constexpr int CK_STRIDE = 32;      // checkpoint stride of the early window sums
constexpr int PART_RING = 32;      // steps of worker partials in flight
constexpr int SLOT_RING = 64;      // published slot records kept
constexpr int HEAD_GROUP = 8;      // lanes per state in the head
constexpr int GRID_MAX_N = GRID_THREADS / HEAD_GROUP;
constexpr int EMPTY_D = 0xffff;
constexpr int TV_ETIMEOUT_DEV = -10;

struct GridParams {
  int G, L, S, Rd, M;
  long long chunk;
  int max_seg;
  unsigned long long w_qd, w_ctil, w_dsel, w_acc, w_itil, w_red, w_bytes;
  unsigned long long h_qtr, h_ctil, h_itil, h_dstar, h_E, h_qd, h_dur, h_dq, h_ptil, h_pv, h_pd, h_pi, h_tail,
      h_red, h_bytes;
  long long timeout;
};

struct GridBufs {
  const int32_t* obs;
  long long T;
  uint32_t* psi;               // (T, N)
  int32_t* path;               // (T)
  double* loglik;              // (1) or null
  long long* slot_ctil;        // [SLOT_RING][N]
  unsigned short* slot_itil;   // [SLOT_RING][N]
  double* slot_dsel;           // [SLOT_RING][N] exact delta[s][argmax i]
  unsigned long long* part;    // [PART_RING][S][3] tagged messages
  double* dstar_g;             // [Rd][N] exact delta ring
  const double* dinit;         // [D][N] initialisation scores
  const double* ck;            // [D][M][N] checkpoints of the early window sums
  const int* seg_first;        // [N]
  const int* seg_count;        // [N]
  const int* seg_base;         // [G-1]
  unsigned* pub;               // number of slots the head has published
  int* abort_flag;
  int* status;
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

__device__ __forceinline__ void grid_fail(const GridBufs& B, int code) {
  atomicExch(B.abort_flag, 1);
  atomicCAS(B.status, 0, code);
}

// Block-wide reduction of an ExactBest; every thread receives the result.
__device__ __forceinline__ ExactBest block_reduce_exact(ExactBest eb, ExactBest* scratch) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
  eb.warp_reduce();
  __syncthreads();
  if (lane == 0) scratch[warp] = eb;
  __syncthreads();
  ExactBest r;
  r.init();
  if (lane < nw) r = scratch[lane];
  r.warp_reduce();
  return r;
}

// ---------------------------------------------------------------------------
// Worker CTA
// ---------------------------------------------------------------------------
__device__ void grid_worker(const ModelView& m, const GridParams& P, const GridBufs& B, unsigned char* sm) {
  const int N = m.N, D = m.D, L = P.L;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int w = blockIdx.x - 1;
  const long long ND = (long long)N * D;
  const long long c_lo = (long long)w * P.chunk;
  const long long c_hi = c_lo + P.chunk < ND ? c_lo + P.chunk : ND;
  if (c_lo >= c_hi) return;  // idle worker: owns no cells, publishes nothing
  const int ja = (int)(c_lo / D), jb = (int)((c_hi - 1) / D);
  const int nseg = jb - ja + 1;
  const int off0 = (int)(c_lo - (long long)ja * D);  // ring slot of the first cell
  const int seg0 = B.seg_base[w];
  const long long T = B.T;
  long long* qd = (long long*)(sm + P.w_qd);
  long long* ctil = (long long*)(sm + P.w_ctil);
  double* dsel = (double*)(sm + P.w_dsel);
  double* acc = (double*)(sm + P.w_acc);
  unsigned short* itil = (unsigned short*)(sm + P.w_itil);
  Top2* red = (Top2*)(sm + P.w_red);  // [max_seg][32]
  ExactBest* ered = (ExactBest*)(sm + P.w_red);
  __shared__ int s_ok;
  __shared__ unsigned s_pub;

  for (long long k = tid; k < (long long)nseg * D; k += blockDim.x) qd[k] = m.qdurT[(size_t)ja * D + k];
  unsigned pub_seen = 0;
  __syncthreads();

  auto seg_range = [&](int s, int& rb, int& re) {
    rb = (s == 0) ? off0 : 0;
    re = (s == nseg - 1) ? (int)(c_hi - (long long)jb * D) : D;
  };

  for (long long t = 1; t < T; ++t) {
    const int tau = (int)(t < D ? t : D);
    const int r0 = (int)((t - 1) % D);
    const long long s_new = t - 1 - L;

    // Intake of the slot record that enters the worker domain (d = L).
    if (s_new >= 0) {
      if (pub_seen < (unsigned)(s_new + 1)) {
        if (tid == 0) {
          unsigned seen = 0;
          s_ok = wait_geq(B.pub, (unsigned)(s_new + 1), seen, B.abort_flag, P.timeout) ? 1 : 0;
          s_pub = seen;
          if (!s_ok) grid_fail(B, TV_ETIMEOUT_DEV);
        }
        __syncthreads();
        if (!s_ok) return;
        pub_seen = s_pub;
      }
      const int r_new = (int)(s_new % D);
      if (tid < nseg) {
        int rb, re;
        seg_range(tid, rb, re);
        if (r_new >= rb && r_new < re) {
          const int j = ja + tid;
          const int c = tid * D + r_new - off0;
          const size_t rec = (size_t)(s_new % SLOT_RING) * N + j;
          ctil[c] = __ldcg(B.slot_ctil + rec);
          itil[c] = __ldcg(B.slot_itil + rec);
          dsel[c] = __ldcg(B.slot_dsel + rec);
        }
      }
    }
    // First step past D: seed the running folds with the reference's
    // newest-first window sums of step D (slot s = r has d = D-1-r then).
    if (t == D + 1) {
      for (int s = 0; s < nseg; ++s) {
        int rb, re;
        seg_range(s, rb, re);
        for (int r = rb + tid; r < re; r += blockDim.x)
          acc[s * D + r - off0] = early_window(m, B.ck, P.M, B.obs, D, D - 1 - r, ja + s);
      }
    }
    __syncthreads();

    // Window fold (t > D) and fixed-point scan over d in [L, tau).
    const int ot = B.obs[t];
    for (int s = 0; s < nseg; ++s) {
      int rb, re;
      seg_range(s, rb, re);
      const int j = ja + s;
      const double emj = m.em[(size_t)ot * N + j];
      Top2 tb;
      tb.init();
      for (int r = rb + tid; r < re; r += blockDim.x) {
        const int c = s * D + r - off0;
        int d = r0 - r;
        if (d < 0) d += D;
        if (t > D) {
          const double a = (d == 0) ? 0.0 : acc[c];
          acc[c] = a + emj;
        }
        if (d >= L && d < tau) tb.push(ctil[c] + qd[s * D + d], d);
      }
      tb.warp_reduce();
      if (lane == 0) red[s * 32 + warp] = tb;
    }
    __syncthreads();

    // Certified exact winner per segment, published as a tagged message.
    if (warp < nseg) {
      const int s = warp;
      const int j = ja + s;
      int rb, re;
      seg_range(s, rb, re);
      Top2 tb;
      tb.init();
      if (lane < (int)(blockDim.x >> 5)) tb = red[s * 32 + lane];
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
          const int i1 = it & 0x7fff;
          const double e = (t > D) ? acc[c1] : early_window(m, B.ck, P.M, B.obs, t, d1, j);
          const double v = (e + dsel[c1]) + (m.trans[(size_t)j * N + i1] + m.durT[(size_t)j * D + d1]);
          eb.v = v; eb.d = d1; eb.i = i1;
        } else {
          const long long thr = tb.b1 - m.margin;
          for (int r = rb + lane; r < re; r += 32) {
            const int c = s * D + r - off0;
            int d = r0 - r;
            if (d < 0) d += D;
            if (d < L || d >= tau) continue;
            if (ctil[c] + qd[s * D + d] < thr) continue;
            const double e = (t > D) ? acc[c] : early_window(m, B.ck, P.M, B.obs, t, d, j);
            const double du = m.durT[(size_t)j * D + d];
            const double* row = B.dstar_g + (size_t)((t - 1 - d) % P.Rd) * N;
            const double* tr = m.trans + (size_t)j * N;
            for (int i = 0; i < N; ++i) eb.offer((e + __ldcg(row + i)) + (tr[i] + du), d, i);
          }
          eb.warp_reduce();
        }
      }
      if (lane == 0) {
        TaggedMsg msg;
        msg_pack(msg, (unsigned)t, eb.v, eb.d == IDX_NONE ? EMPTY_D : eb.d, eb.d == IDX_NONE ? 0 : eb.i);
        msg_store(B.part + ((size_t)(t % PART_RING) * P.S + seg0 + s) * 3, msg);
      }
    }
    __syncthreads();
  }

  // Tail at t = T-1: exhaustive exact scan of the worker's cells with the
  // survival function (src/hsmm.cu:101-137), one partial per segment.
  {
    const long long t = T - 1;
    const int tau = (int)(t < D ? t : D);
    const int r0 = t >= 1 ? (int)((t - 1) % D) : 0;
    for (int s = 0; s < nseg; ++s) {
      int rb, re;
      seg_range(s, rb, re);
      const int j = ja + s;
      ExactBest eb;
      eb.init();
      for (int r = rb + tid; r < re; r += blockDim.x) {
        const int c = s * D + r - off0;
        int d = r0 - r;
        if (d < 0) d += D;
        if (d < L || d >= tau) continue;
        const double E = (t > D) ? acc[c] : early_window(m, B.ck, P.M, B.obs, t, d, j);
        const double e = E + m.survT[(size_t)j * D + d];
        const double* row = B.dstar_g + (size_t)((t - 1 - d) % P.Rd) * N;
        const double* tr = m.trans + (size_t)j * N;
        for (int i = 0; i < N; ++i) eb.offer((e + __ldcg(row + i)) + tr[i], d, i);
      }
      eb = block_reduce_exact(eb, ered);
      if (tid == 0) {
        TaggedMsg msg;
        msg_pack(msg, (unsigned)T, eb.v, eb.d == IDX_NONE ? EMPTY_D : eb.d, eb.d == IDX_NONE ? 0 : eb.i);
        msg_store(B.part + ((size_t)(T % PART_RING) * P.S + seg0 + s) * 3, msg);
      }
    }
  }
}

// ---------------------------------------------------------------------------
// Head CTA
// ---------------------------------------------------------------------------
__device__ void grid_head(const ModelView& m, const GridParams& P, const GridBufs& B, unsigned char* sm) {
  const int N = m.N, D = m.D, L = P.L, S = P.S;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int g = tid / HEAD_GROUP, gl = tid % HEAD_GROUP;
  const unsigned gmask = 0xffu << ((lane / HEAD_GROUP) * HEAD_GROUP);
  const long long T = B.T;
  long long* qtr = (long long*)(sm + P.h_qtr);        // [N][N]
  long long* ctil_h = (long long*)(sm + P.h_ctil);    // [L][N]
  unsigned short* itil_h = (unsigned short*)(sm + P.h_itil);
  double* dstar_h = (double*)(sm + P.h_dstar);        // [L+1][N]
  double* E_h = (double*)(sm + P.h_E);                // [L][N]
  long long* qd_h = (long long*)(sm + P.h_qd);        // [N][L]
  double* dur_h = (double*)(sm + P.h_dur);            // [N][L]
  long long* dq = (long long*)(sm + P.h_dq);
  long long* ptil = (long long*)(sm + P.h_ptil);
  double* pv = (double*)(sm + P.h_pv);
  int* pd = (int*)(sm + P.h_pd);
  int* pi = (int*)(sm + P.h_pi);
  double* tail = (double*)(sm + P.h_tail);
  __shared__ int s_fail;

  for (int k = tid; k < N * N; k += blockDim.x) qtr[k] = m.qtr[k];
  for (int k = tid; k < N * L; k += blockDim.x) {
    const int j = k / L, d = k % L;
    qd_h[k] = m.qdurT[(size_t)j * D + d];
    dur_h[k] = m.durT[(size_t)j * D + d];
  }
  for (int j = tid; j < N; j += blockDim.x) {
    const double d0 = B.dinit[j];
    dstar_h[j] = d0;
    B.dstar_g[j] = d0;
    dq[j] = quantize(d0, m.scale);
    ptil[j] = m.qem[(size_t)B.obs[0] * N + j];
    B.psi[j] = pack_psi(0, 0);
  }
  if (tid == 0) s_fail = 0;
  const int j = g;  // this group's state (N <= GRID_MAX_N)
  const bool has_j = j < N;
  double di_cur = 0.0;
  if (has_j && 1 < D) di_cur = __ldcg(B.dinit + (size_t)1 * N + j);
  __syncthreads();

  for (long long t = 1; t < T; ++t) {
    const int tau = (int)(t < D ? t : D);
    const int hl = tau < L ? tau : L;
    // Worker partials of this step: issue the loads first, check them after
    // the matvec has hidden their latency.
    TaggedMsg pm;
    if (tid < S) msg_load(B.part + ((size_t)(t % PART_RING) * S + tid) * 3, pm);
    const int ot = B.obs[t];
    double di_next = 0.0;
    if (has_j && t + 1 < D) di_next = __ldcg(B.dinit + (size_t)(t + 1) * N + j);

    // Phase B: matvec for slot s = t-1, its publication, P(t), window sums.
    if (has_j) {
      Top2 tb;
      tb.init();
      for (int i = gl; i < N; i += HEAD_GROUP) tb.push(qtr[j * N + i] + dq[i], i);
#pragma unroll
      for (int o = HEAD_GROUP / 2; o > 0; o >>= 1) {
        const long long ob1 = __shfl_xor_sync(gmask, tb.b1, o);
        const long long ob2 = __shfl_xor_sync(gmask, tb.b2, o);
        const int ox1 = __shfl_xor_sync(gmask, tb.x1, o);
        tb.merge(ob1, ox1, ob2);
      }
      const double emt = m.em[(size_t)ot * N + j];
      if (t > D) {
        // E_t[d] = E_{t-1}[d-1] + em_t, E_t[0] = 0 + em_t (src/hsmm.cu:298-310)
        const double old = gl < L ? E_h[gl * N + j] : 0.0;
        const double prev = __shfl_up_sync(gmask, old, 1, HEAD_GROUP);
        if (gl < L) E_h[gl * N + j] = (gl == 0 ? 0.0 : prev) + emt;
      } else if (gl == 0) {
        // newest-first rebuild (src/hsmm.cu:311-322)
        double gsum = emt;
        E_h[j] = gsum;
        for (int d = 1; d < hl; ++d) {
          gsum = gsum + m.em[(size_t)B.obs[t - d] * N + j];
          E_h[d * N + j] = gsum;
        }
      }
      if (gl == 0) {
        const long long c = tb.b1 - ptil[j];
        const bool amb = (tb.b1 - tb.b2) <= m.margin;
        const unsigned short itv = (unsigned short)(tb.x1 | (amb ? 0x8000 : 0));
        const int hrow = (int)((t - 1) % L);
        ctil_h[hrow * N + j] = c;
        itil_h[hrow * N + j] = itv;
        const size_t rec = (size_t)((t - 1) % SLOT_RING) * N + j;
        B.slot_ctil[rec] = c;
        B.slot_itil[rec] = itv;
        B.slot_dsel[rec] = dstar_h[(size_t)((t - 1) % (L + 1)) * N + tb.x1];
        ptil[j] += m.qem[(size_t)ot * N + j];
      }
    }
    if (tid < S) {
      if (!msg_wait(B.part + ((size_t)(t % PART_RING) * S + tid) * 3, (unsigned)t, pm, B.abort_flag, P.timeout)) {
        grid_fail(B, TV_ETIMEOUT_DEV);
        s_fail = 1;
      } else {
        msg_unpack(pm, pv[tid], pd[tid], pi[tid]);
      }
    }
    __syncthreads();
    if (s_fail) return;
    if (tid == 0) {
      __threadfence();
      st_release_u32(B.pub, (unsigned)t);  // slots 0..t-1 are published
    }

    // Phase C: the head's candidates d < L, certified; merge; finalise.
    if (has_j) {
      Top2 tb;
      tb.init();
      for (int d = gl; d < hl; d += HEAD_GROUP) tb.push(ctil_h[(int)((t - 1 - d) % L) * N + j] + qd_h[j * L + d], d);
#pragma unroll
      for (int o = HEAD_GROUP / 2; o > 0; o >>= 1) {
        const long long ob1 = __shfl_xor_sync(gmask, tb.b1, o);
        const long long ob2 = __shfl_xor_sync(gmask, tb.b2, o);
        const int ox1 = __shfl_xor_sync(gmask, tb.x1, o);
        tb.merge(ob1, ox1, ob2);
      }
      const int d1 = tb.x1;
      const unsigned short it = itil_h[(int)((t - 1 - d1) % L) * N + j];
      const bool amb = (it & 0x8000) || ((tb.b1 - tb.b2) <= m.margin);
      ExactBest eb;
      eb.init();
      if (!amb) {
        const int i1 = it & 0x7fff;
        eb.v = (E_h[d1 * N + j] + dstar_h[(size_t)((t - 1 - d1) % (L + 1)) * N + i1]) +
               (m.trans[(size_t)j * N + i1] + dur_h[j * L + d1]);
        eb.d = d1;
        eb.i = i1;
      } else {
        const long long thr = tb.b1 - m.margin;
        for (int d = gl; d < hl; d += HEAD_GROUP) {
          if (ctil_h[(int)((t - 1 - d) % L) * N + j] + qd_h[j * L + d] < thr) continue;
          const double e = E_h[d * N + j];
          const double du = dur_h[j * L + d];
          const double* row = dstar_h + (size_t)((t - 1 - d) % (L + 1)) * N;
          const double* tr = m.trans + (size_t)j * N;
          for (int i = 0; i < N; ++i) eb.offer((e + row[i]) + (tr[i] + du), d, i);
        }
#pragma unroll
        for (int o = HEAD_GROUP / 2; o > 0; o >>= 1) {
          const double ov = __shfl_xor_sync(gmask, eb.v, o);
          const int od = __shfl_xor_sync(gmask, eb.d, o);
          const int oi = __shfl_xor_sync(gmask, eb.i, o);
          eb.offer(ov, od, oi);
        }
      }
      const int k0 = B.seg_first[j], k1 = k0 + B.seg_count[j];
      for (int k = k0; k < k1; ++k)
        if (pd[k] != EMPTY_D) eb.offer(pv[k], pd[k], pi[k]);
      if (gl == 0) {
        double fin;
        uint32_t wv;
        // t < D: the induction result replaces the initialisation score only
        // when strictly larger (src/hsmm.cu:353-358).
        if (t >= D || eb.v > di_cur) {
          fin = eb.v;
          wv = pack_psi(eb.d, eb.i);
        } else {
          fin = di_cur;
          wv = pack_psi((int)t, 0);
        }
        dstar_h[(size_t)(t % (L + 1)) * N + j] = fin;
        B.dstar_g[(size_t)(t % P.Rd) * N + j] = fin;
        dq[j] = quantize(fin, m.scale);
        B.psi[(size_t)t * N + j] = wv;
      }
    }
    di_cur = di_next;
    __syncthreads();
  }

  // Tail at t = T-1 (src/hsmm.cu:101-137).
  {
    const long long t = T - 1;
    const int tau = (int)(t < D ? t : D);
    const int hl = tau < L ? tau : L;
    TaggedMsg pm;
    if (tid < S) {
      msg_load(B.part + ((size_t)(T % PART_RING) * S + tid) * 3, pm);
      if (!msg_wait(B.part + ((size_t)(T % PART_RING) * S + tid) * 3, (unsigned)T, pm, B.abort_flag, P.timeout)) {
        grid_fail(B, TV_ETIMEOUT_DEV);
        s_fail = 1;
      } else {
        msg_unpack(pm, pv[tid], pd[tid], pi[tid]);
      }
    }
    __syncthreads();
    if (s_fail) return;
    if (has_j) {
      ExactBest eb;
      eb.init();
      for (int d = gl; d < hl; d += HEAD_GROUP) {
        const double e = E_h[d * N + j] + m.survT[(size_t)j * D + d];
        const double* row = dstar_h + (size_t)((t - 1 - d) % (L + 1)) * N;
        const double* tr = m.trans + (size_t)j * N;
        for (int i = 0; i < N; ++i) eb.offer((e + row[i]) + tr[i], d, i);
      }
#pragma unroll
      for (int o = HEAD_GROUP / 2; o > 0; o >>= 1) {
        const double ov = __shfl_xor_sync(gmask, eb.v, o);
        const int od = __shfl_xor_sync(gmask, eb.d, o);
        const int oi = __shfl_xor_sync(gmask, eb.i, o);
        eb.offer(ov, od, oi);
      }
      const int k0 = B.seg_first[j], k1 = k0 + B.seg_count[j];
      for (int k = k0; k < k1; ++k)
        if (pd[k] != EMPTY_D) eb.offer(pv[k], pd[k], pi[k]);
      if (gl == 0) {
        if (eb.d == IDX_NONE) { eb.d = 0; eb.i = 0; }
        tail[j] = eb.v;
        B.psi[(size_t)t * N + j] = pack_psi(eb.d, eb.i);
      }
    }
    __syncthreads();
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

__global__ void __launch_bounds__(GRID_THREADS, 1) grid_decode_kernel(ModelView m, GridParams P, GridBufs B) {
  extern __shared__ __align__(16) unsigned char smem[];
  if (ld_relaxed_i32(B.abort_flag)) return;  // rejected observations
  if (blockIdx.x == 0)
    grid_head(m, P, B, smem);
  else
    grid_worker(m, P, B, smem);
}

}  // namespace tv
