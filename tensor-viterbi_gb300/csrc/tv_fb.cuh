// tv_fb.cuh -- the forward-backward E step of HSMM training on the GPU.
//
// The reference's training step is hsmmlearn's EM fit
// (hsmmlearn/hsmmlearn/hsmm.py:181-305), whose E step is FBImpl
// (hsmmlearn/hsmmlearn/_hsmm/src/FBImpl.cpp): Guedon's scaled forward and
// backward recursions for an explicit-duration HSMM, then the expected
// duration counts eta.  These kernels compute the same arrays with the same
// formulas; one CTA runs one sequence.  fb_kernel (any J) uses a warp per
// state (lanes over the durations u) for the O(J*M) sums of a step and a
// thread per state for the O(J) normalisation and transition sums, which
// keep the reference's sequential order (j, i or k ascending);
// fb_small_kernel (J <= 32) shortens the chain of a step (below).
//
// The products of likelihood ratios r_s = pdf[j][s] / N[s] over a segment
// are kept per state and duration (in a ring indexed by the segment's first
// (forward) or last (backward) step, or in registers), and multiplied by the
// new ratio every step (one multiply per cell, like the decoder's window
// folds), instead of being rebuilt for every u as the reference does; and
// the sums over u are lane partials reduced by shuffles (or, for the window
// sums of fb_small_kernel, exactly in 64-bit integers).  Both change the
// association of some products and sums, so results agree with the
// reference to rounding (relative differences of order 1e-13 on the tests'
// sequences), not bit for bit.  The backward right-censoring product s is
// formed in the reference's order.
//
// Censoring 0 (none) and 1 (right censoring, the fit's default) are
// supported; the reference's left-censoring variant (2) is not.
//
// This file is included by tv_host.cu.
#pragma once

namespace tv {

struct FbArgs {
  int censoring, tau, J, M;
  const double* d;    // (J, M) duration pmf, entry u-1 = P(duration u)
  const double* p;    // (J, J) [from][to]
  const double* pi;   // (J)
  const double* pdf;  // (J, tau)
  double *F, *L, *G, *L1, *N, *Norm, *eta;  // outputs, hsmmlearn's layouts
  double* S;          // (J, tau) scratch: StateIn
  double* D;          // (J, M+1) scratch: survival D[j][u] = sum_{v >= u} d[j][v]
  double* ring;       // (2, J, M) scratch when the rings do not fit shared memory
                      // (fb_small_kernel: the first two of (3, J, M))
  int rings_in_smem;
  double* R;          // (J, tau) scratch of fb_small_kernel: r = pdf / N
  double* A;          // (J, tau) scratch of fb_small_kernel: sum_{i != j} p[i][j] F[i][t]
  double* Q;          // (J, tau) scratch of fb_small_kernel<K > 0>: L1 / F (the backward
                      // window's new entry), for the eta kernels
  double* part;       // (J, nchunks, M) scratch: eta sums of the chunks of t
  long long chunk;    // steps of t per chunk
  int nchunks;
  int* status;        // 0, or 1 where the reference throws var_nonpositive_exception
};

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

__global__ void __launch_bounds__(1024) fb_kernel(FbArgs a) {
  extern __shared__ __align__(16) unsigned char fsm[];
  const int J = a.J, M = a.M, tau = a.tau;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5, nw = blockDim.x >> 5;
  const bool right = a.censoring == 1;
  double* Pf = a.rings_in_smem ? (double*)fsm : a.ring;  // [J][M] forward ring, by segment start s % M
  double* Pb = Pf + (size_t)J * M;                         // [J][M] backward ring, by segment end e % M
  __shared__ int s_bad;
  __shared__ double s_N;
  auto at = [&](double* x, int j, long long t) -> double& { return x[(size_t)j * tau + t]; };
  auto atc = [&](const double* x, int j, long long t) -> double { return x[(size_t)j * tau + t]; };
  auto dd = [&](int j, int u) -> double { return a.d[(size_t)j * M + (u - 1)]; };       // d[j][u], u = 1..M
  auto DD = [&](int j, int u) -> double { return u <= M ? a.D[(size_t)j * (M + 1) + u] : 0.0; };
  auto pp = [&](int i, int j) -> double { return a.p[(size_t)i * J + j]; };

  if (tid == 0) s_bad = 0;
  // CalcStoreD (dCalc.cpp:5-30): each sum from v = u upwards, as there
  for (int j = warp; j < J; j += nw)
    for (int u = lane + 1; u <= M; u += 32) {
      double x = 0;
      for (int v = u; v <= M; ++v) x += dd(j, v);
      a.D[(size_t)j * (M + 1) + u] = x;
    }
  for (int j = warp; j < J; j += nw)
    for (int u = lane + 1; u <= M; u += 32) a.eta[(size_t)j * M + (u - 1)] = 0.0;
  __syncthreads();

  // ---- forward recursion (FBImpl.cpp:62-140) ----
  for (int t = 0; t < tau; ++t) {
    for (int j = tid; j < J; j += blockDim.x)
      at(a.Norm, j, t) = t == 0 ? atc(a.pdf, j, 0) * a.pi[j]
                                : atc(a.pdf, j, t) * (at(a.S, j, t) - at(a.F, j, t - 1) + at(a.Norm, j, t - 1));
    __syncthreads();
    if (tid == 0) {
      double n = 0;
      for (int j = 0; j < J; ++j) n += at(a.Norm, j, t);
      a.N[t] = n;
      s_N = n;
      if (!(n > 0)) s_bad = 1;
    }
    __syncthreads();
    if (s_bad) break;
    const double Nt = s_N;
    for (int j = tid; j < J; j += blockDim.x) at(a.Norm, j, t) /= Nt;
    // F[j][t] = sum_u P(t-u+1..t) * dur(u) * StateIn[j][t-u+1] (the segment
    // that started at s = 0 takes pi instead); the last step takes the
    // survival D instead of d
    const bool last = t == tau - 1;
    const int umax = min(t + 1, M);
    for (int j = warp; j < J; j += nw) {
      const double r = atc(a.pdf, j, t) / Nt;
      double* P = Pf + (size_t)j * M;
      double part = 0.0;
      for (int u = lane + 1; u <= umax; u += 32) {
        const int s = t - u + 1;
        const int slot = s % M;
        const double ob = (u == 1) ? r : P[slot] * r;
        P[slot] = ob;
        const double du = last ? DD(j, u) : dd(j, u);
        part += (s > 0) ? ob * du * at(a.S, j, s) : ob * du * a.pi[j];
      }
      const double f = warp_sum(part);
      if (lane == 0) {
        at(a.F, j, t) = f;
        if (!(f > 0)) s_bad = 1;
      }
    }
    __syncthreads();
    if (s_bad) break;
    if (t < tau - 1)
      for (int j = tid; j < J; j += blockDim.x) {
        double x = 0;
        for (int i = 0; i < J; ++i) x += pp(i, j) * at(a.F, i, t);
        at(a.S, j, t + 1) = x;
      }
    __syncthreads();
  }
  if (s_bad) {
    if (tid == 0) *a.status = 1;
    return;
  }

  // ---- backward recursion (FBImpl.cpp:142-178) with eta (:231-270) ----
  for (int j = tid; j < J; j += blockDim.x) at(a.L, j, tau - 1) = at(a.F, j, tau - 1);
  __syncthreads();
  for (int t = tau - 2; t >= 0; --t) {
    const int span = tau - 1 - t;  // steps after t
    const int umax = min(span, M);
    for (int j = warp; j < J; j += nw) {
      const double r = atc(a.pdf, j, t + 1) / a.N[t + 1];
      double* Q = Pb + (size_t)j * M;
      // A = sum_{i != j} p[i][j] F[i][t] (the eta weight of this step)
      double A = 0;
      for (int i = 0; i < J; ++i)
        if (i != j) A += pp(i, j) * at(a.F, i, t);
      double part = 0.0;
      for (int u = lane + 1; u <= umax; u += 32) {
        const int e = t + u;  // the segment t+1..e
        const int slot = e % M;
        const double ob = (u == 1) ? r : Q[slot] * r;
        Q[slot] = ob;
        const double h = (u < span) ? at(a.L1, j, e) * ob * dd(j, u) / at(a.F, j, e) : ob * DD(j, span);
        part += h;
        // eta: H term for u <= span - 1, right-censored term for u = span
        if (u <= span - 1) a.eta[(size_t)j * M + (u - 1)] += A * h;
      }
      // right censoring: u >= span, the product over t+1..tau-1 (the
      // reference's s, formed backwards: the ring entry of e = tau-1)
      if (right && span <= M) {
        __syncwarp();  // the lane that owns u = span wrote the entry
        const double s_t = Q[(tau - 1) % M];
        for (int u = lane + 1; u <= M; u += 32)
          if (u >= span) a.eta[(size_t)j * M + (u - 1)] += A * (s_t * dd(j, u));
      }
      const double g = warp_sum(part);
      if (lane == 0) at(a.G, j, t + 1) = g;
    }
    __syncthreads();
    for (int j = tid; j < J; j += blockDim.x) {
      double x = 0;
      for (int k = 0; k < J; ++k) x += at(a.G, k, t + 1) * pp(j, k);
      x *= at(a.F, j, t);
      at(a.L1, j, t) = x;
      at(a.L, j, t) = x + at(a.L, j, t + 1) - at(a.G, j, t + 1) * at(a.S, j, t + 1);
    }
    __syncthreads();
  }

  // eta: the segment that starts at t = 0 (FBImpl.cpp:252-266)
  for (int j = warp; j < J; j += nw)
    for (int u = lane + 1; u <= M; u += 32) {
      if (!(right || u <= tau - 1)) continue;
      double r = dd(j, u) * a.pi[j];
      if (u <= tau - 1) {
        for (int v = 1; v <= u; ++v) r *= atc(a.pdf, j, u - v) / a.N[u - v];
        r *= at(a.L1, j, u - 1) / at(a.F, j, u - 1);
      } else {
        for (int v = 1; v <= tau; ++v) r *= atc(a.pdf, j, tau - v) / a.N[tau - v];
      }
      a.eta[(size_t)j * M + (u - 1)] += r;
    }
  if (tid == 0) *a.status = 0;
}

// Sum over the aligned group of g lanes (g a power of two <= 32); every lane
// of the warp takes part.
__device__ __forceinline__ double group_sum(double v, int g) {
  for (int o = g >> 1; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// Sum over the aligned group of g lanes (g a power of two <= 32) of finite
// doubles, formed in 64-bit integers: each lane's significand is aligned to
// the group's largest exponent (with five bits of headroom for 32 terms) and
// truncated there, the integers are summed exactly by shuffles, and the sum
// is converted to double once, so the FP64 unit runs one conversion instead
// of log2(g) dependent adds.  Error: below 2^-52 of the largest term's
// magnitude (the same order as a tree of double adds).  A group holding an
// infinity or NaN is summed with double adds.
__device__ __forceinline__ double fixed_group_sum(double v, int g) {
  const unsigned full = 0xffffffffu;
  if (__any_sync(full, ((__double_as_longlong(v) >> 52) & 0x7ff) == 0x7ff)) return group_sum(v, g);
  const long long b = __double_as_longlong(v);
  const int e = (int)((b >> 52) & 0x7ff);
  const long long m = (b & 0xfffffffffffffLL) | (e ? (1LL << 52) : 0LL);
  const int ee = e ? e : 1;  // subnormals share the smallest normal exponent
  int emax = ee;
  for (int o = g >> 1; o > 0; o >>= 1) emax = max(emax, __shfl_xor_sync(full, emax, o));
  const int sh = emax - ee;
  long long f = sh >= 58 ? 0LL : (m << 5) >> sh;  // units of 2^(emax - 1080)
  if (b < 0) f = -f;
  for (int o = g >> 1; o > 0; o >>= 1) f += __shfl_xor_sync(full, f, o);
  // f * 2^(emax - 1080): exact exponent arithmetic when the result is normal
  const double c = __ll2double_rn(f);
  const long long cb = __double_as_longlong(c);
  const int ce = (int)((cb >> 52) & 0x7ff) + emax - 1080;
  if (f == 0) return 0.0;
  if (ce >= 1 && ce <= 2046) return __longlong_as_double((cb & ~(0x7ffLL << 52)) | ((long long)ce << 52));
  return ldexp(c, emax - 1080);
}

// Durations a lane of fb_small_kernel<K, MAXT> holds in registers:
// u = lane + 1 + 32k for k < K, so K blocks of 32 cover a window of up to
// 32K durations.  MAXT is the launch bound (32 J threads): 512 leaves the
// register window room without spilling.
constexpr int FB_REG_BLOCKS = 4;

// fb_small_kernel: the same E step for J <= 32 states, one warp per state.
// A step is a chain of dependent FP64 operations, shuffles and barriers on
// one SM (a sequence has no other parallelism), and GB300's FP64 units have
// a long dependent latency, so the kernel keeps that chain short:
//   forward:  warp 0 (a lane per state) forms the normaliser N[t] with one
//             shuffle reduction and one division, then the ratios
//             r = pdf * (1/N); warp j keeps, per duration u of the window,
//             W(u) = P(t-u+1..t) * StateIn(t-u+1) (the segment that starts at
//             t-u+1), which is W(u-1) of step t-1 times r: with K > 0 the
//             entries live in registers (lane + 32k holds u = lane + 1 + 32k)
//             and move up one duration per step by warp shuffles; with K = 0
//             in a shared-memory ring indexed by the segment start.  F is the
//             sum of W(u) * dur(u): fused multiply-adds, then a warp
//             reduction in 64-bit integers (fixed_group_sum: ten warps of
//             double-add trees would occupy the SM's FP64 unit);
//             groups of lanes (a power of two >= J per state) form
//             StateIn[j][t+1], and the eta weight A[j][t] = sum_{i != j}
//             p[i][j] F[i][t] where the backward pass reads it (every step
//             with K = 0; the last M steps with K > 0).
//   backward: warp j keeps V(u) = Q(t+1..t+u) * L1(t+u) / F(t+u) for the
//             segment that ends at t+u, V(u-1) of step t+1 times r, the same
//             way, so a segment term is V(u) * d(u); groups of lanes form
//             L1 = F * sum_k G[k] p[j][k] and L, and L1 / F is taken as that
//             sum.  Eta: with K = 0 the accumulators take A * V (and the
//             right-censored terms A * s, s formed in the reference's order)
//             without the factor d(u), applied once at the end; with K > 0
//             only the right-censored terms are taken here, L1 / F is stored
//             per step, and fb_eta_chunk_kernel / fb_eta_final_kernel form the
//             A * V terms off this chain and finish eta.
// The ratios of the forward pass are kept for the backward pass.
// Products, the sums over u, i, k and j, fused multiply-adds and the
// divisions associate differently from the reference (which sums in order
// and divides each term), which moves results by rounding only.
template <int K, int MAXT>
__global__ void __launch_bounds__(MAXT) fb_small_kernel(FbArgs a) {
  extern __shared__ __align__(16) unsigned char fsm[];
  const int J = a.J, M = a.M, tau = a.tau;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5, nw = blockDim.x >> 5;
  const bool right = a.censoring == 1;
  const int jw = warp;  // this warp's state in the window passes (nw == J)
  // K = 0: the window rings and eta accumulators (shared memory when they
  // fit, else global scratch and eta itself)
  double* rings = a.rings_in_smem ? (double*)fsm : a.ring;
  double* Wf = rings;                          // [J][M] forward W, by segment start % M
  double* Vb = Wf + (size_t)J * M;             // [J][M] backward V, by segment end % M
  double* Et = a.rings_in_smem ? Vb + (size_t)J * M : a.eta;
  __shared__ double s_r[32], s_F[32], s_S[32], s_G[32], s_q[32];
  __shared__ int s_bad;
  auto at = [&](double* x, int j, long long t) -> double& { return x[(size_t)j * tau + t]; };
  auto atc = [&](const double* x, int j, long long t) -> double { return x[(size_t)j * tau + t]; };
  auto dd = [&](int j, int u) -> double { return __ldg(a.d + (size_t)j * M + (u - 1)); };
  auto DD = [&](int j, int u) -> double { return u <= M ? a.D[(size_t)j * (M + 1) + u] : 0.0; };
  auto pp = [&](int i, int j) -> double { return __ldg(a.p + (size_t)i * J + j); };
  // lane groups for the J x J sums: Gs lanes per state, 32 / Gs states a warp
  int Gs = 1;
  while (Gs < J) Gs <<= 1;
  const int per_warp = 32 / Gs;
  const int gj = warp * per_warp + lane / Gs;  // this lane's state in the grouped sums
  const int gi = lane % Gs;                     // and its i (or k)
  const bool glead = gi == 0 && gj < J;
  constexpr int KR = K > 0 ? K : 1;
  double dk[KR], wk[KR], vk[KR], ek[KR];  // K > 0: d(u), W(u), V(u), eta accumulator of u = lane + 1 + 32k
#pragma unroll
  for (int k = 0; k < KR; ++k) {
    const int u = lane + 1 + 32 * k;
    dk[k] = (K > 0 && jw < J && u <= M) ? dd(jw, u) : 0.0;
    wk[k] = vk[k] = ek[k] = 0.0;
  }

  if (tid == 0) s_bad = 0;
  for (int j = warp; j < J; j += nw)
    for (int u = lane + 1; u <= M; u += 32) {
      double x = 0;
      for (int v = u; v <= M; ++v) x += dd(j, v);
      a.D[(size_t)j * (M + 1) + u] = x;
      if (K == 0) Et[(size_t)j * M + (u - 1)] = 0.0;
    }
  if (tid < 32) s_S[tid] = s_q[tid] = 0.0;
  __syncthreads();

  // ---- forward ----
  // Values read from global memory on a step's chain are loaded one step
  // ahead into registers (a global load costs hundreds of clocks).
  double Fprev = 0.0, Nmprev = 0.0, Scur = 0.0;  // warp 0, lane j: F[j][t-1], Norm[j][t-1], StateIn[j][t]
  double pdf_cur = (warp == 0 && lane < J) ? atc(a.pdf, lane, 0) : 0.0;
  for (int t = 0; t < tau; ++t) {
    if (warp == 0) {
      const bool has = lane < J;
      const double pdf_nx = (has && t + 1 < tau) ? atc(a.pdf, lane, t + 1) : 0.0;
      double raw = 0.0;
      if (has) raw = t == 0 ? pdf_cur * a.pi[lane] : pdf_cur * (Scur - Fprev + Nmprev);
      const double n = group_sum(raw, Gs);
      const double inv = 1.0 / n;
      if (has) {
        const double nm = raw * inv;
        at(a.Norm, lane, t) = nm;
        Nmprev = nm;
        const double r = pdf_cur * inv;
        s_r[lane] = r;
        at(a.R, lane, t) = r;
      }
      if (lane == 0) {
        a.N[t] = n;
        if (!(n > 0)) s_bad = 1;
      }
      pdf_cur = pdf_nx;
    }
    __syncthreads();
    if (s_bad) break;
    const bool last = t == tau - 1;
    const int umax = min(t + 1, M);
    if (jw < J) {
      const double r = s_r[jw];
      // a new segment start takes StateIn (or pi for s = 0)
      const double sin = t > 0 ? s_S[jw] : a.pi[jw];
      double part = 0.0;
      if constexpr (K > 0) {
        double carry = 0.0;
#pragma unroll
        for (int k = 0; k < K; ++k) {
          if (32 * k < umax) {
            // W(u) of step t is W(u-1) of step t-1 times r
            const double up = __shfl_up_sync(0xffffffffu, wk[k], 1);
            const double top = __shfl_sync(0xffffffffu, wk[k], 31);
            const double prev = lane == 0 ? (k == 0 ? sin : carry) : up;
            carry = top;
            wk[k] = prev * r;
            const int u = lane + 1 + 32 * k;
            if (u <= umax) part = __fma_rn(wk[k], last ? DD(jw, u) : dk[k], part);
          }
        }
      } else {
        double* W = Wf + (size_t)jw * M;
        for (int u = lane + 1; u <= umax; u += 32) {
          const int slot = (t - u + 1) % M;
          const double w = (u == 1 ? sin : W[slot]) * r;
          W[slot] = w;
          part = __fma_rn(w, last ? DD(jw, u) : dd(jw, u), part);
        }
      }
      const double f = fixed_group_sum(part, 32);
      if (lane == 0) {
        s_F[jw] = f;
        at(a.F, jw, t) = f;
        if (!(f > 0)) s_bad = 1;
      }
    }
    __syncthreads();
    if (s_bad) break;
    if (t < tau - 1 && warp * per_warp < J) {
      const double pr = (gj < J && gi < J) ? pp(gi, gj) * s_F[gi] : 0.0;
      // the eta weight A[t] is read by the backward pass only while
      // tau - 1 - t <= M with K > 0 (fb_eta_chunk_kernel forms the rest
      // itself, in the same order), at every step with K = 0
      if (K == 0 || t >= tau - 1 - M) {
        double sv = pr, av = gi != gj ? pr : 0.0;
        for (int o = Gs >> 1; o > 0; o >>= 1) {
          sv += __shfl_xor_sync(0xffffffffu, sv, o);
          av += __shfl_xor_sync(0xffffffffu, av, o);
        }
        if (glead) {
          s_S[gj] = sv;
          at(a.S, gj, t + 1) = sv;
          at(a.A, gj, t) = av;
        }
      } else {
        double sv = pr;
        for (int o = Gs >> 1; o > 0; o >>= 1) sv += __shfl_xor_sync(0xffffffffu, sv, o);
        if (glead) {
          s_S[gj] = sv;
          at(a.S, gj, t + 1) = sv;
        }
      }
    }
    __syncthreads();
    if (warp == 0 && lane < J) {
      Fprev = s_F[lane];
      Scur = s_S[lane];
    }
  }
  if (s_bad) {
    if (tid == 0) *a.status = 1;
    return;
  }

  // ---- backward ----
  // warp j: r = pdf/N of step t+1 and the eta weight of step t, loaded
  // during step t+1; the group leader of state j: F[j][t], StateIn[j][t+1]
  // likewise, and L[j][t+1] from the previous step
  double r_nx = 0.0, A_nx = 0.0, s_tail = 1.0;
  if (jw < J && tau >= 2) {
    r_nx = at(a.R, jw, tau - 1);
    A_nx = at(a.A, jw, tau - 2);
  }
  double Lnext = 0.0, f_nx = 0.0, st_nx = 0.0;
  if (glead) {
    Lnext = at(a.F, gj, tau - 1);
    at(a.L, gj, tau - 1) = Lnext;
    if (tau >= 2) {
      f_nx = at(a.F, gj, tau - 2);
      st_nx = at(a.S, gj, tau - 1);
    }
  }
  __syncthreads();
  for (int t = tau - 2; t >= 0; --t) {
    const int span = tau - 1 - t;
    const int umax = min(span, M);
    const double r = r_nx, A = A_nx;
    if (jw < J && t >= 1) {
      r_nx = at(a.R, jw, t);
      A_nx = at(a.A, jw, t - 1);
    }
    if (jw < J) {
      // the reference's s: r[tau-1] * r[tau-2] * ... * r[t+1], read only
      // while span <= M (the tail term and the right-censored eta terms)
      if (span <= M) s_tail = s_tail * r;
      const double q = s_q[jw];  // L1(t+1) / F(t+1)
      double part = 0.0;
      if constexpr (K > 0) {
        double carry = 0.0;
#pragma unroll
        for (int k = 0; k < K; ++k) {
          if (32 * k < umax) {
            // V(u) of step t is V(u-1) of step t+1 times r
            const double up = __shfl_up_sync(0xffffffffu, vk[k], 1);
            const double top = __shfl_sync(0xffffffffu, vk[k], 31);
            const double prev = lane == 0 ? (k == 0 ? q : carry) : up;
            carry = top;
            vk[k] = prev * r;
            const int u = lane + 1 + 32 * k;
            if (u < span && u <= M) {
              part = __fma_rn(vk[k], dk[k], part);  // its eta term A * V: fb_eta_chunk_kernel
            } else if (u == span) {
              part = __fma_rn(s_tail, DD(jw, span), part);
            }
          }
        }
        if (right && span <= M) {
#pragma unroll
          for (int k = 0; k < K; ++k) {
            const int u = lane + 1 + 32 * k;
            if (u >= span && u <= M) ek[k] = __fma_rn(A, s_tail, ek[k]);
          }
        }
      } else {
        double* V = Vb + (size_t)jw * M;
        double* E = Et + (size_t)jw * M;
        for (int u = lane + 1; u <= umax; u += 32) {
          if (u < span) {
            const int slot = (t + u) % M;
            const double v = (u == 1 ? q : V[slot]) * r;
            V[slot] = v;
            part = __fma_rn(v, dd(jw, u), part);
            E[u - 1] = __fma_rn(A, v, E[u - 1]);
          } else {
            part = __fma_rn(s_tail, DD(jw, span), part);
          }
        }
        if (right && span <= M)
          for (int u = lane + 1; u <= M; u += 32)
            if (u >= span) E[u - 1] = __fma_rn(A, s_tail, E[u - 1]);
      }
      const double g = fixed_group_sum(part, 32);
      if (lane == 0) {
        s_G[jw] = g;
        at(a.G, jw, t + 1) = g;
      }
    }
    __syncthreads();
    const double f_t = f_nx, st1 = st_nx;
    if (glead && t >= 1) {
      f_nx = at(a.F, gj, t - 1);
      st_nx = at(a.S, gj, t);
    }
    if (warp * per_warp < J) {
      double sv = (gj < J && gi < J) ? s_G[gi] * pp(gj, gi) : 0.0;
      for (int o = Gs >> 1; o > 0; o >>= 1) sv += __shfl_xor_sync(0xffffffffu, sv, o);
      if (glead) {
        const double l1 = sv * f_t;
        at(a.L1, gj, t) = l1;
        const double lv = l1 + Lnext - s_G[gj] * st1;
        at(a.L, gj, t) = lv;
        Lnext = lv;
        s_q[gj] = sv;
        if (K > 0) at(a.Q, gj, t) = sv;
      }
    }
    __syncthreads();
  }

  // K > 0: eta's right-censored terms (A * s) go to eta; fb_eta_chunk_kernel
  // and fb_eta_final_kernel add the window terms and finish it.
  if constexpr (K > 0) {
    if (jw < J) {
#pragma unroll
      for (int k = 0; k < K; ++k) {
        const int u = lane + 1 + 32 * k;
        if (u <= M) a.eta[(size_t)jw * M + (u - 1)] = ek[k];
      }
    }
    if (tid == 0) *a.status = 0;
    return;
  }
  // eta = d(u) * (accumulated A * V and A * s) + the segment that starts at
  // t = 0 (FBImpl.cpp:252-266)
  if (jw < J) {
    const int j = jw;
    for (int u = lane + 1; u <= M; u += 32) {
      double w = Et[(size_t)j * M + (u - 1)] * dd(j, u);
      if (right || u <= tau - 1) {
        double r = dd(j, u) * a.pi[j];
        if (u <= tau - 1) {
          for (int v = 1; v <= u; ++v) r *= atc(a.pdf, j, u - v) / a.N[u - v];
          r *= at(a.L1, j, u - 1) / at(a.F, j, u - 1);
        } else {
          for (int v = 1; v <= tau; ++v) r *= atc(a.pdf, j, tau - v) / a.N[tau - v];
        }
        w += r;
      }
      a.eta[(size_t)j * M + (u - 1)] = w;
    }
  }
  if (tid == 0) *a.status = 0;
}

// The eta term of the segment that starts at t = 0 (FBImpl.cpp:252-266).
__device__ __forceinline__ double fb_eta_initial(const FbArgs& a, int j, int u) {
  const int tau = a.tau, M = a.M;
  double r = __ldg(a.d + (size_t)j * M + (u - 1)) * a.pi[j];
  if (u <= tau - 1) {
    for (int v = 1; v <= u; ++v) r *= a.pdf[(size_t)j * tau + (u - v)] / a.N[u - v];
    r *= a.L1[(size_t)j * tau + (u - 1)] / a.F[(size_t)j * tau + (u - 1)];
  } else {
    for (int v = 1; v <= tau; ++v) r *= a.pdf[(size_t)j * tau + (tau - v)] / a.N[tau - v];
  }
  return r;
}

// fb_eta_chunk_kernel: the window terms of eta, off the backward chain.
// eta[j][u] collects A[j][t] * V_t(u) over the steps t with t + u <= tau - 2,
// where V_t(u) = r[t+1] * V_{t+1}(u-1) and V_t(1) = r[t+1] * Q[t+1] is the
// backward window of fb_small_kernel (the same products in the same order,
// from the ratios R and the entries Q it stored).  One warp per (chunk of t,
// state): it rebuilds the window from M - 1 steps above its chunk (an entry
// for segment end e enters at t = e - 1), then accumulates over the chunk,
// the window in registers moved by shuffles as in the backward pass.
template <int K>
__global__ void __launch_bounds__(32) fb_eta_chunk_kernel(FbArgs a) {
  if (*a.status != 0) return;
  const int j = blockIdx.y, c = blockIdx.x, lane = threadIdx.x;
  const int tau = a.tau, M = a.M;
  const long long t0 = (long long)c * a.chunk;
  const long long t1 = min((long long)tau - 1, t0 + a.chunk);  // t in [t0, t1), t <= tau - 2
  double vk[K], acc[K];
#pragma unroll
  for (int k = 0; k < K; ++k) vk[k] = acc[k] = 0.0;
  const int J = a.J;
  const double* R = a.R + (size_t)j * tau;
  const double* Qr = a.Q + (size_t)j * tau;
  // the eta weight A[t] = sum_{i != j} p[i][j] F[i][t], lane i the term of
  // state i: the same products and the same xor tree as the forward pass's
  // lane groups (lanes past the group add zeros), so the same values
  const bool has_i = lane < J && lane != j;
  const double pij = has_i ? __ldg(a.p + (size_t)lane * J + j) : 0.0;
  const double* Fi = a.F + (size_t)(lane < J ? lane : 0) * tau;
  const long long ts = min((long long)tau - 2, t1 + M - 2);
  // a step's ratio, entry and F term, loaded a step ahead
  double r_nx = 0.0, q_nx = 0.0, f_nx = 0.0;
  if (ts >= t0) {
    r_nx = R[ts + 1];
    q_nx = ts + 1 <= tau - 2 ? Qr[ts + 1] : 0.0;
    f_nx = has_i ? Fi[ts] : 0.0;
  }
  for (long long t = ts; t >= t0; --t) {
    const double r = r_nx, q = q_nx, f = f_nx;
    if (t - 1 >= t0) {
      r_nx = R[t];
      q_nx = t <= tau - 2 ? Qr[t] : 0.0;
      f_nx = has_i ? Fi[t - 1] : 0.0;
    }
    double carry = 0.0;
#pragma unroll
    for (int k = 0; k < K; ++k) {
      const double up = __shfl_up_sync(0xffffffffu, vk[k], 1);
      const double top = __shfl_sync(0xffffffffu, vk[k], 31);
      const double prev = lane == 0 ? (k == 0 ? q : carry) : up;
      carry = top;
      vk[k] = prev * r;
    }
    if (t < t1) {
      const double A = warp_sum(has_i ? pij * f : 0.0);
#pragma unroll
      for (int k = 0; k < K; ++k) {
        const int u = lane + 1 + 32 * k;
        if (u <= M && t + u <= tau - 2) acc[k] = __fma_rn(A, vk[k], acc[k]);
      }
    }
  }
#pragma unroll
  for (int k = 0; k < K; ++k) {
    const int u = lane + 1 + 32 * k;
    if (u <= M) a.part[((size_t)j * a.nchunks + c) * M + (u - 1)] = acc[k];
  }
}

// fb_eta_final_kernel: eta = d(u) * (right-censored terms + the chunks' window
// terms, chunks in order) + the term of the segment that starts at t = 0.
__global__ void fb_eta_final_kernel(FbArgs a) {
  if (*a.status != 0) return;
  const int j = blockIdx.x, M = a.M;
  const bool right = a.censoring == 1;
  for (int u = threadIdx.x + 1; u <= M; u += blockDim.x) {
    double w = 0.0;
    for (int c = 0; c < a.nchunks; ++c) w += a.part[((size_t)j * a.nchunks + c) * M + (u - 1)];
    w = (a.eta[(size_t)j * M + (u - 1)] + w) * __ldg(a.d + (size_t)j * M + (u - 1));
    if (right || u <= a.tau - 1) w += fb_eta_initial(a, j, u);
    a.eta[(size_t)j * M + (u - 1)] = w;
  }
}

}  // namespace tv
