// tv_floor.cuh -- the per-step latency floor of the grid decoder's head, and
// the latency of one cross-SM message round trip (diagnostics for the
// benchmark's roofline; no reference counterpart).
//
// The grid decoder's period is set by the head CTA's critical lanes: each
// step needs the previous step's whole score row before its N x N matvec can
// start, so the recurrence is a serial chain of one matvec, one hand-over,
// one exact score and one barrier per step.  floor_chain_kernel runs that
// chain alone on one SM, with nothing else on it: the packed coarse matvec of
// slot t-1 with the head's layout, loads and two max chains (the upper half on
// its own warps when the plan splits it, handed over at the pair barrier),
// the exact d = 0 score (two dependent FP64 adds on the argmax's row), its
// fixed-point value and coarse re-pack against the previous step's base, and
// the step barrier.  Its clocks per step are what the head's period would be
// with every other role (certification, the helpers' merges, the intake of the
// workers' partials, the stores) free.
//
// xsm_roundtrip_kernel bounces a tagged 64-bit word between CTA 0 and the last
// CTA of a cooperative grid of one CTA per SM, with the decoder's own tagged
// stores and bounded polling loads: the latency a head-worker message pays,
// hidden in the decoder by the workers' L-step lead.
//
// fp64_issue_kernel measures one SM's FP64 unit, the bound of the
// forward-backward kernel (one sequence runs on one SM): with several warps
// of threads each running eight independent fused multiply-add chains, the
// SM's FP64 issue rate; with one warp and one chain, the dependent latency of
// one FP64 instruction.
//
// This file is included by tv_host.cu after tv_grid.cuh.
#pragma once

namespace tv {

__global__ void fp64_issue_kernel(int independent, long long iters, const double* __restrict__ in, double* sink,
                                  unsigned long long* clk) {
  const double y = in[8], z = in[9];
  double a0 = in[0], a1 = in[1], a2 = in[2], a3 = in[3], a4 = in[4], a5 = in[5], a6 = in[6], a7 = in[7];
  __syncthreads();
  const long long t0 = clock64();
  if (independent) {
    for (long long i = 0; i < iters; ++i) {
      a0 = __fma_rn(a0, y, z); a1 = __fma_rn(a1, y, z); a2 = __fma_rn(a2, y, z); a3 = __fma_rn(a3, y, z);
      a4 = __fma_rn(a4, y, z); a5 = __fma_rn(a5, y, z); a6 = __fma_rn(a6, y, z); a7 = __fma_rn(a7, y, z);
    }
  } else {
    for (long long i = 0; i < iters; ++i) a0 = __fma_rn(a0, y, z);
  }
  const long long t1 = clock64();
  sink[threadIdx.x] = a0 + a1 + a2 + a3 + a4 + a5 + a6 + a7;
  if ((threadIdx.x & 31) == 0) atomicMax(clk, (unsigned long long)(t1 - t0));
}

__global__ void floor_chain_kernel(int N, int Np, int split, long long steps, const double* __restrict__ trans,
                                   double scale, int sh, long long* out) {
  extern __shared__ __align__(16) unsigned char fsm[];
  const int Qs = Np + 4;
  int* Qcp = (int*)fsm;                                              // [N][Qs]
  int* dqcp = Qcp + (size_t)N * Qs;                                  // [2][Np]
  long long* dq = (long long*)(dqcp + 2 * Np);                       // [2][N] (Np even: 8-byte aligned)
  double* dstar = (double*)(dq + 2 * N);                             // [2][N]
  double* trh = dstar + 2 * N;                                       // [N][N]
  int2* xch = (int2*)(trh + (size_t)N * N);                          // [Np]
  int* ambf = (int*)(xch + Np);                                      // [Np] coarse certification
  const int tid = threadIdx.x;
  const int cs = (N + 31) / 32 * 32;
  const int csb = split ? cs : 0;
  const int Nh = split ? (Np / 16) * 8 : Np;
  for (int k = tid; k < N * Np; k += blockDim.x) {
    const int j = k / Np, i = k % Np;
    if (i < N) {
      const long long q = __double2ll_rn(trans[(size_t)j * N + i] * scale);
      Qcp[j * Qs + i] = coarse_of(q, sh) * 128 + (127 - i);
    } else {
      Qcp[j * Qs + i] = INT_MIN;
    }
  }
  for (int k = tid; k < N * N; k += blockDim.x) trh[k] = trans[k];
  for (int k = tid; k < 2 * Np; k += blockDim.x) dqcp[k] = 0;
  for (int j = tid; j < N; j += blockDim.x) {
    dstar[j] = -0.5 * j;
    dq[j] = __double2ll_rn(dstar[j] * scale);
  }
  __syncthreads();
  for (int j = tid; j < N; j += blockDim.x) dqcp[j] = coarse_of(dq[j] - dq[0], sh) * 128;
  __syncthreads();
  long long c0 = clock64();
  if (tid < cs) {
    const int j = tid;
    const double e0 = -1.0 - 0.001 * j, du0 = -0.5;
    for (long long t = 1; t <= steps; ++t) {
      const int cur = (int)(t & 1), prv = cur ^ 1;
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
      if (split) named_sync(BAR_PAIR0 + (tid >> 5), 64);
      if (j < N) {
        if (split) {
          const int2 o = xch[j];
          const int lo = min(b1, o.x);
          b1 = max(b1, o.x);
          b2 = max(max(b2, o.y), lo);
        }
        const int ifine = 127 - (b1 & 127);
        ambf[j] = ((b1 >> 7) - (b2 >> 7)) <= 2;  // the head's coarse certification test
        const double V0 = (e0 + dstar[prv * N + ifine]) + (trh[(size_t)j * N + ifine] + du0);
        const long long q = __double2ll_rn(V0 * scale);
        dstar[cur * N + j] = V0;
        dq[cur * N + j] = q;
        dqcp[cur * Np + j] = coarse_of(q - dq[prv * N], sh) * 128;
      }
      named_sync(BAR_STEP, cs + csb);
    }
  } else if (tid < cs + csb) {
    const int jb = tid - cs;
    for (long long t = 1; t <= steps; ++t) {
      const int prv = (int)(t & 1) ^ 1;
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
      named_sync(BAR_STEP, cs + csb);
    }
  }
  __syncthreads();
  if (tid == 0) {
    out[0] = clock64() - c0;
    double s = 0.0;
    long long a = 0;
    for (int j = 0; j < N; ++j) {
      s += dstar[(int)(steps & 1) * N + j];
      a += ambf[j];
    }
    out[1] = (long long)s + a;  // keeps the chain's results live
  }
}

// One CTA per SM (the launch's shared memory keeps two apart); thread 0 of
// CTA 0 and of the last CTA exchange `iters` tagged words.  Every wait gives
// up after `limit` clocks or when the other side raised *status.
__global__ void xsm_roundtrip_kernel(unsigned long long* words, int iters, long long limit, long long* out,
                                     int* status) {
  const int G = gridDim.x;
  if (threadIdx.x != 0 || G < 2 || (blockIdx.x != 0 && blockIdx.x != G - 1)) return;
  unsigned smid;
  asm volatile("mov.u32 %0, %%smid;" : "=r"(smid));
  unsigned long long v;
  if (blockIdx.x == 0) {
    const long long c0 = clock64();
    for (int k = 1; k <= iters; ++k) {
      tagged64_store(words, (unsigned)k, (unsigned long long)k);
      if (!tagged64_load(words + 2, (unsigned)k, v, status, limit)) {
        atomicExch(status, 1);
        return;
      }
    }
    out[0] = clock64() - c0;
    out[1] = smid;
  } else {
    for (int k = 1; k <= iters; ++k) {
      if (!tagged64_load(words, (unsigned)k, v, status, limit)) {
        atomicExch(status, 1);
        return;
      }
      tagged64_store(words + 2, (unsigned)k, v);
    }
    out[2] = smid;
  }
}

}  // namespace tv
