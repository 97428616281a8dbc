// tv_cta.cuh -- one CTA decodes one sequence at a time; a persistent grid
// walks a queue of sequences.  This is the batched form (many sequences in one
// launch) and the single-sequence form for small N*D windows.
//
// Per sequence the CTA keeps the D-deep score window in shared memory (or in
// a per-CTA global scratch slab when it does not fit):
//   qd    [N][D] int64   quantised duration log-pmf, d-contiguous
//   ctil  [N][D] int64   ring over predecessor end s (slot s % D):
//                        C(s, j) = max_i(qtrans[j][i] + qdelta[s][i]) - P(s, j)
//                        where P is the running fixed-point emission prefix
//   itil  [N][D] u16     argmax i of that max; bit 15 set when its runner-up
//                        is inside the margin (the i-order is not certified)
//   acc   [N][D] double  exact emission window sums E_t for slot s: the value
//                        the reference holds in EMISSION_PROBS[t-1-s]
//   dstar [D+1][N] double exact scores delta[s][i] (reference delta_t values)
//   qtr   [N][N] int64   quantised transition log-probs
// Per step t the candidate score of (j, d) with predecessor slot s = t-1-d is
//   P(t, j) + C(s, j) + qd[j][d]
// and P(t, j) is common to all d of a state, so the scan is one int64 add and
// a top-2 update per cell.  The exact score of the winner is then formed in
// the reference's association
//   (E_t[d][j] + delta[s][i]) + (trans[j][i] + dur[j][d])   (src/hsmm.cu:341-346)
#pragma once
#include "tv_device.cuh"

namespace tv {

struct ModelView {
  int N, O, D;
  const double* em;       // (O, N) exact log emission
  const double* trans;    // (N, N) exact, [to j][from i]
  const double* start;    // (N)
  const double* durT;     // (N, D) exact log duration pmf, [j][d]
  const double* survT;    // (N, D) exact log survival, [j][d]
  const long long* qem;   // (O, N) fixed point
  const long long* qtr;   // (N, N) fixed point
  const long long* qdurT; // (N, D) fixed point
  double scale;           // 2^f
  long long margin;       // certified near-tie margin, fixed-point units
};

struct BatchView {
  const int32_t* obs;     // concatenated observations
  const int64_t* off;     // (n_seq + 1) offsets
  int32_t* path;          // concatenated paths
  double* loglik;         // (n_seq) or null
  uint32_t* psi;          // concatenated (T_k, N) back-pointer words
  int* status;            // (n_seq)
  int* next;              // work-queue counter, zero at launch
  const int* order;       // queue order (longest first), or null for 0..n_seq-1
  int n_seq;
};

struct CtaLayout {
  // byte offsets inside the per-CTA work area
  unsigned long long o_qd, o_ctil, o_acc, o_dstar, o_itil, o_qtr, o_dq, o_ptil, o_tail;
  unsigned long long bytes;
  int in_smem;
  int qd_global;  // qd read from the model's table in global memory (through L1), not copied per CTA
};

__host__ __device__ inline unsigned long long tv_align(unsigned long long x) { return (x + 15ull) & ~15ull; }

// qd_global: leave the quantised duration table (8 N D bytes, the same for
// every CTA) out of the work area, so that more CTAs share an SM's shared
// memory; the scan then reads it from global memory, cached in L1.
__host__ inline CtaLayout make_cta_layout(int N, int D, bool qd_global = false) {
  CtaLayout L{};
  unsigned long long o = 0;
  const unsigned long long nd = (unsigned long long)N * D;
  L.qd_global = qd_global ? 1 : 0;
  L.o_qd = o;    if (!qd_global) o = tv_align(o + nd * 8);
  L.o_ctil = o;  o = tv_align(o + nd * 8);
  L.o_acc = o;   o = tv_align(o + nd * 8);
  L.o_dstar = o; o = tv_align(o + (unsigned long long)(D + 1) * N * 8);
  L.o_itil = o;  o = tv_align(o + nd * 2);
  L.o_qtr = o;   o = tv_align(o + (unsigned long long)N * N * 8);
  L.o_dq = o;    o = tv_align(o + (unsigned long long)N * 8);
  L.o_ptil = o;  o = tv_align(o + (unsigned long long)N * 8);
  L.o_tail = o;  o = tv_align(o + (unsigned long long)N * 8);
  L.bytes = o;
  L.in_smem = 0;
  return L;
}

// One step's exact winner for state j when the fixed-point scan is not
// certified: every candidate whose fixed-point score is within `margin` of
// the best is re-scored exactly; the rest cannot reach the maximum.
__device__ __forceinline__ ExactBest rescore_state(const ModelView& m, int j, long long t, int tau,
                                                   int r0, long long thr, const long long* qd,
                                                   const long long* ctil, const double* acc,
                                                   const double* dstar, int lane) {
  const int N = m.N, D = m.D;
  ExactBest eb;
  eb.init();
  for (int d = lane; d < tau; d += 32) {
    int r = r0 - d;
    if (r < 0) r += D;
    const long long v = ctil[(size_t)j * D + r] + qd[(size_t)j * D + d];
    if (v >= thr) {
      const double e = acc[(size_t)j * D + r];
      const double du = m.durT[(size_t)j * D + d];
      const long long s = t - 1 - d;
      const double* row = dstar + (size_t)(s % (D + 1)) * N;
      const double* tr = m.trans + (size_t)j * N;
      for (int i = 0; i < N; ++i) eb.offer((e + row[i]) + (tr[i] + du), d, i);
    }
  }
  eb.warp_reduce();
  return eb;
}

template <int NTHREADS>
__global__ void __launch_bounds__(NTHREADS) cta_decode_kernel(ModelView m, BatchView b, CtaLayout L,
                                                              unsigned char* scratch) {
  extern __shared__ __align__(16) unsigned char smem[];
  constexpr int NWARPS = NTHREADS / 32;
  const int N = m.N, D = m.D;
  const int lane = threadIdx.x & 31;
  const int warp = threadIdx.x >> 5;
  unsigned char* base = L.in_smem ? smem : scratch + (size_t)blockIdx.x * L.bytes;
  long long* qd_w = (long long*)(base + L.o_qd);
  const long long* qd = L.qd_global ? m.qdurT : qd_w;
  long long* ctil = (long long*)(base + L.o_ctil);
  double* acc = (double*)(base + L.o_acc);
  double* dstar = (double*)(base + L.o_dstar);
  unsigned short* itil = (unsigned short*)(base + L.o_itil);
  long long* qtr = (long long*)(base + L.o_qtr);
  long long* dq = (long long*)(base + L.o_dq);
  long long* ptil = (long long*)(base + L.o_ptil);
  double* tail = (double*)(base + L.o_tail);
  __shared__ int s_seq;
  __shared__ int s_bad;
  // fraction bits f of the fixed point (scale = 2^f)
  const int qf = (int)((__double_as_longlong(m.scale) >> 52) & 0x7ff) - 1023;
  constexpr long long RESCORED = 1LL << 62;  // flag of a parked winner re-scored in phase 2
  int G = 1;  // lanes per state in the transition matvec
  while (G < 32 && G * 4 < N) G <<= 1;

  // Model tables shared by every sequence of the batch.
  if (!L.qd_global)
    for (size_t k = threadIdx.x; k < (size_t)N * D; k += NTHREADS) qd_w[k] = m.qdurT[k];
  for (size_t k = threadIdx.x; k < (size_t)N * N; k += NTHREADS) qtr[k] = m.qtr[k];

  for (;;) {
    __syncthreads();
    if (threadIdx.x == 0) {
      const int k = atomicAdd(b.next, 1);
      s_seq = k < b.n_seq ? (b.order ? b.order[k] : k) : b.n_seq;
    }
    __syncthreads();
    const int seq = s_seq;
    if (seq >= b.n_seq) break;
    const long long T0 = b.off[seq];
    const long long T = b.off[seq + 1] - T0;
    const int32_t* obs = b.obs + T0;
    uint32_t* psi = b.psi + (size_t)T0 * N;
    int32_t* path = b.path + T0;

    // Observations may come straight from device memory: range-check them
    // before any table lookup; a bad sequence is reported and skipped.
    if (threadIdx.x == 0) s_bad = 0;
    __syncthreads();
    for (long long t = threadIdx.x; t < T; t += NTHREADS)
      if ((unsigned)obs[t] >= (unsigned)m.O) s_bad = 1;
    __syncthreads();
    if (s_bad || T < D) {
      if (threadIdx.x == 0) b.status[seq] = -3;
      continue;
    }

    // Initialisation, t < D: delta[t][j] = (dur[j][t] + start[j]) + E0[t][j],
    // E0 the oldest-first running sum of the emissions (src/hsmm.cu:274-290).
    // Ring slot t % (D+1) of dstar is t itself for t < D.
    for (int j = threadIdx.x; j < N; j += NTHREADS) {
      double e = 0.0;
      const double sj = m.start[j];
      for (int d = 0; d < D; ++d) {
        e = e + m.em[(size_t)obs[d] * N + j];
        dstar[(size_t)d * N + j] = (m.durT[(size_t)j * D + d] + sj) + e;
      }
      psi[j] = pack_psi(0, 0);
      dq[j] = quantize(dstar[j], m.scale);
      ptil[j] = m.qem[(size_t)obs[0] * N + j];
    }
    __syncthreads();

    // Ring positions kept incrementally (a 64-bit remainder by a runtime
    // divisor is a long dependent integer sequence): r0 = (t-1) % D, the slot
    // of s = t-1 in ctil/itil/acc, and rt = t % (D+1), the row of step t in
    // dstar.  The observation of step t+1 is loaded a step ahead.
    int r0 = 0, rt = 1 % (D + 1);
    int ot_nx = T > 1 ? obs[1] : 0;
    for (long long t = 1; t < T; ++t) {
      const int tau = (int)(t < D ? t : D);
      const int ot = ot_nx;
      if (t + 1 < T) ot_nx = obs[t + 1];

      // Phase 0 (t <= D): the reference rebuilds the window sums newest-first,
      // E_t[d] = E_t[d-1] + em_{t-d} (src/hsmm.cu:311-322).  One chain per
      // state; slot of d is t-1-d (no wrap while t <= D).
      if (t <= D) {
        for (int j = threadIdx.x; j < N; j += NTHREADS) {
          double g = m.em[(size_t)ot * N + j];
          acc[(size_t)j * D + (t - 1)] = g;
          for (int d = 1; d < tau; ++d) {
            g = g + m.em[(size_t)obs[t - d] * N + j];
            acc[(size_t)j * D + (t - 1 - d)] = g;
          }
        }
      }

      // Phase 1: max-plus transition matvec for the newest predecessor slot
      // s = t-1, and the emission prefix P(t) = P(t-1) + qem[obs[t]].
      // A group of G lanes per state (about four predecessors a lane, G a
      // power of two up to a warp), so a small N takes few warps and few
      // shuffle rounds.
      for (int j0 = warp * (32 / G); j0 < N; j0 += NWARPS * (32 / G)) {
        const int j = j0 + lane / G, u = lane % G;
        Top2 tb;
        tb.init();
        if (j < N)
          for (int i = u; i < N; i += G) tb.push(qtr[(size_t)j * N + i] + dq[i], i);
        for (int o = G >> 1; o > 0; o >>= 1) {
          const long long ob1 = __shfl_xor_sync(0xffffffffu, tb.b1, o);
          const long long ob2 = __shfl_xor_sync(0xffffffffu, tb.b2, o);
          const int ox1 = __shfl_xor_sync(0xffffffffu, tb.x1, o);
          tb.merge(ob1, ox1, ob2);
        }
        if (u == 0 && j < N) {
          ctil[(size_t)j * D + r0] = tb.b1 - ptil[j];
          const bool amb = (tb.b1 - tb.b2) <= m.margin;
          itil[(size_t)j * D + r0] = (unsigned short)(tb.x1 | (amb ? 0x8000 : 0));
          ptil[j] += m.qem[(size_t)ot * N + j];
        }
      }
      __syncthreads();

      // Phase 2: per state, the window update (t > D: E_t[d] = E_{t-1}[d-1] +
      // em_t with E_t[0] = 0 + em_t, src/hsmm.cu:298-310), the fixed-point
      // scan over d and the certified exact winner.
      for (int j = warp; j < N; j += NWARPS) {
        const double emj = m.em[(size_t)ot * N + j];
        Top2 tb;
        tb.init();
        if (t > D) {
          for (int d = lane; d < tau; d += 32) {
            int r = r0 - d;
            if (r < 0) r += D;
            const size_t k = (size_t)j * D + r;
            const double a = (d == 0) ? 0.0 : acc[k];
            acc[k] = a + emj;
            tb.push(ctil[k] + qd[(size_t)j * D + d], d);
          }
        } else {
          for (int d = lane; d < tau; d += 32) {
            const int r = r0 - d;
            tb.push(ctil[(size_t)j * D + r] + qd[(size_t)j * D + d], d);
          }
        }
        tb.warp_reduce();
        __syncwarp();

        // The certified argmax (d1, i1) is parked in dq[j] (dq is not read
        // again before phase 3 overwrites it); an ambiguous state is re-scored
        // exactly here by its warp and parked with its exact value in tail[j].
        const int d1 = tb.x1;
        int r1 = r0 - d1;
        if (r1 < 0) r1 += D;
        const unsigned short it = itil[(size_t)j * D + r1];
        const bool amb = (it & 0x8000) || ((tb.b1 - tb.b2) <= m.margin);
        if (!amb) {
          if (lane == 0) dq[j] = (long long)pack_psi(d1, it & 0x7fff);
        } else {
          const ExactBest eb = rescore_state(m, j, t, tau, r0, tb.b1 - m.margin, qd, ctil, acc, dstar, lane);
          if (lane == 0) {
            tail[j] = eb.value();
            dq[j] = (long long)pack_psi(eb.d, eb.i) | RESCORED;
          }
        }
      }
      __syncthreads();

      // Phase 3: one lane per state, the exact score of each certified winner
      // (src/hsmm.cu:341-346), the replacement rule for t < D (:353-358), the
      // new delta row and back-pointers.  One lane per state keeps the FP64
      // work of a step in few warp instructions (GB300 charges a warp-wide
      // FP64 instruction the same pipe time however few lanes are active).
      for (int j = threadIdx.x; j < N; j += NTHREADS) {
        const long long w = dq[j];
        const int bd = (int)((w >> 16) & 0xffff), bi = (int)(w & 0xffff);
        double vbest;
        if (w & RESCORED) {
          vbest = tail[j];
        } else {
          int r1 = r0 - bd;
          if (r1 < 0) r1 += D;
          int rs = rt - 1 - bd;  // (t-1-bd) % (D+1), 0 <= bd < D
          if (rs < 0) rs += D + 1;
          const double e = acc[(size_t)j * D + r1];
          const double dp = dstar[(size_t)rs * N + bi];
          vbest = (e + dp) + (m.trans[(size_t)j * N + bi] + m.durT[(size_t)j * D + bd]);
        }
        double* slot = dstar + (size_t)rt * N + j;
        // For t < D the induction result replaces the initialisation value
        // only when strictly larger (src/hsmm.cu:353-358).
        double fin;
        uint32_t pw;
        if (t >= D || vbest > *slot) {
          fin = vbest;
          pw = pack_psi(bd, bi);
        } else {
          fin = *slot;
          pw = pack_psi((int)t, 0);
        }
        *slot = fin;
        dq[j] = fixed_from_double(fin, qf);
        psi[(size_t)t * N + j] = pw;
      }
      __syncthreads();
      r0 = r0 + 1 == D ? 0 : r0 + 1;
      rt = rt + 1 == D + 1 ? 0 : rt + 1;
    }

    // Tail adjustment at t = T-1 (src/hsmm.cu:101-137): survival in place of
    // the duration pmf, association ((E + surv) + delta) + trans, exhaustive
    // exact scan, unconditional overwrite of row T-1.
    {
      const long long t = T - 1;
      const int tau = (int)(t < D ? t : D);
      const int r0 = t >= 1 ? (int)((t - 1) % D) : 0;
      for (int j = warp; j < N; j += NWARPS) {
        ExactBest eb;
        eb.init();
        for (int d = lane; d < tau; d += 32) {
          int r = r0 - d;
          if (r < 0) r += D;
          const double e = acc[(size_t)j * D + r] + m.survT[(size_t)j * D + d];
          const long long s = t - 1 - d;
          const double* row = dstar + (size_t)(s % (D + 1)) * N;
          const double* tr = m.trans + (size_t)j * N;
          for (int i = 0; i < N; ++i) eb.offer((e + row[i]) + tr[i], d, i);
        }
        eb.warp_reduce();
        if (lane == 0) {
          if (eb.d == IDX_NONE) { eb.d = 0; eb.i = 0; }
          tail[j] = eb.value();
          psi[(size_t)t * N + j] = pack_psi(eb.d, eb.i);
        }
      }
    }
    __syncthreads();

    // Backtrace (src/hsmm.cu:139-170) by warp 0: lane 0 follows the
    // back-pointers, the warp fills each segment.
    if (warp == 0) {
      int cur = 0;
      double best = tail[0];
      for (int n = 1; n < N; ++n)
        if (tail[n] > best) { best = tail[n]; cur = n; }
      long long t = T - 1;
      int bad = 0;
      while (t >= 0) {
        uint32_t w = 0;
        if (lane == 0) w = psi[(size_t)t * N + cur];
        w = __shfl_sync(0xffffffffu, w, 0);
        const long long len = (long long)(w >> 16) + 1;
        const int prev = (int)(w & 0xffffu);
        if (len > t + 1 || prev >= N) { bad = 1; break; }
        for (long long k = t - len + 1 + lane; k <= t; k += 32) path[k] = cur;
        t -= len;
        cur = prev;
      }
      if (lane == 0) {
        if (b.loglik) b.loglik[seq] = best;
        b.status[seq] = bad ? -8 : 0;
      }
    }
  }
}

}  // namespace tv
