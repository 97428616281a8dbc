// tv_device.cuh -- device-side building blocks shared by the decode kernels.
//
// Scores are compared in int64 fixed point (value * 2^f, f chosen per decode
// on the host).  GB300 issues FP64 at 1/64 of the FP32 rate, so the per-cell
// max-plus scan runs on the integer pipes; FP64 is kept for the values the
// reference defines bit for bit (the emission window sums and the winners'
// scores).  A candidate is only trusted when it beats every other one by more
// than the certified margin; otherwise the candidates inside the margin are
// re-scored exactly in FP64 with the reference's association and tie order.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

namespace tv {

// Below every reachable fixed-point score (|score| < 2^61 by the choice of f),
// and far enough from INT64_MIN that b1 - b2 never overflows.
constexpr long long QNEG = -(1LL << 62);
constexpr int IDX_NONE = 0x7fffffff;

// Back-pointer word: (d << 16) | i, where d+1 is the segment length and i the
// previous state.  N and D are limited to 65536.
__device__ __forceinline__ uint32_t pack_psi(int d, int i) {
  return ((uint32_t)d << 16) | (uint32_t)i;
}

// Running best / second best of a fixed-point scan with the index of the
// best.  Inside one lane indices arrive in increasing order, so a strict '>'
// keeps the lowest index of an exact tie.
struct Top2 {
  long long b1;
  long long b2;
  int x1;
  __device__ __forceinline__ void init() { b1 = QNEG; b2 = QNEG; x1 = IDX_NONE; }
  __device__ __forceinline__ void push(long long v, int x) {
    const bool take = v > b1;
    const long long lose = take ? b1 : v;
    b2 = lose > b2 ? lose : b2;
    if (take) { b1 = v; x1 = x; }
  }
  // Merge another lane's state; equal best values keep the lower index.
  __device__ __forceinline__ void merge(long long ob1, int ox1, long long ob2) {
    const bool take = (ob1 > b1) || (ob1 == b1 && ox1 < x1);
    const long long lose = take ? b1 : ob1;
    long long s = b2 > ob2 ? b2 : ob2;
    s = s > lose ? s : lose;
    if (take) { b1 = ob1; x1 = ox1; }
    b2 = s;
  }
  // Butterfly reduction: every lane ends with the warp-wide result.
  __device__ __forceinline__ void warp_reduce() {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      const long long ob1 = __shfl_xor_sync(0xffffffffu, b1, o);
      const long long ob2 = __shfl_xor_sync(0xffffffffu, b2, o);
      const int ox1 = __shfl_xor_sync(0xffffffffu, x1, o);
      merge(ob1, ox1, ob2);
    }
  }
};

// Order-preserving int64 image of a double: comparing keys as signed integers
// orders finite values and -inf as the doubles compare (-0 is mapped to +0 so
// that they tie, as in IEEE).  GB300 issues FP64 at 1/64 of the FP32 rate, so
// exact comparisons run on the integer pipes through these keys.
__device__ __forceinline__ long long order_key(double v) {
  long long b = __double_as_longlong(v);
  if (b == (long long)0x8000000000000000ULL) b = 0;
  return b ^ ((b >> 63) & 0x7fffffffffffffffLL);
}
__device__ __forceinline__ double key_value(long long k) {
  return __longlong_as_double(k ^ ((k >> 63) & 0x7fffffffffffffffLL));
}
constexpr long long KEY_NEG_INF = (long long)0x800fffffffffffffULL;  // order_key(-inf)

// Exact candidate in the reference's order: the larger value wins, then the
// lower d, then the lower i (the d-outer / i-inner strict '>' scan of
// src/hsmm.cu:340-350).
struct ExactBest {
  long long k;  // order_key of the value
  int d;
  int i;
  __device__ __forceinline__ void init() { k = KEY_NEG_INF; d = IDX_NONE; i = IDX_NONE; }
  __device__ __forceinline__ double value() const { return key_value(k); }
  __device__ __forceinline__ void set(double v, int od, int oi) { k = order_key(v); d = od; i = oi; }
  __device__ __forceinline__ bool better_key(long long ok, int od, int oi) const {
    return (ok > k) || (ok == k && (od < d || (od == d && oi < i)));
  }
  __device__ __forceinline__ void offer_key(long long ok, int od, int oi) {
    if (better_key(ok, od, oi)) { k = ok; d = od; i = oi; }
  }
  __device__ __forceinline__ void offer(double v, int od, int oi) { offer_key(order_key(v), od, oi); }
  __device__ __forceinline__ void warp_reduce() {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      const long long ok = __shfl_xor_sync(0xffffffffu, k, o);
      const int od = __shfl_xor_sync(0xffffffffu, d, o);
      const int oi = __shfl_xor_sync(0xffffffffu, i, o);
      offer_key(ok, od, oi);
    }
  }
};

__device__ __forceinline__ long long quantize(double x, double scale) {
  return __double2ll_rn(x * scale);
}

// round-half-even(x * 2^f) from the bits of x, on the integer pipes; equal to
// quantize(x, 2^f) for every finite x whose scaled value fits in int64.
__device__ __forceinline__ long long fixed_from_double(double x, int f) {
  const unsigned long long bits = (unsigned long long)__double_as_longlong(x);
  const int e = (int)((bits >> 52) & 0x7ff);
  if (e == 0) return 0;  // zero or subnormal: |x * 2^f| < 1/2
  const long long M = (long long)((bits & 0xfffffffffffffull) | (1ull << 52));
  const int sh = e - 1075 + f;
  long long q;
  if (sh >= 0) {
    q = M << sh;
  } else if (sh < -54) {
    q = 0;
  } else {
    const int r = -sh;
    q = M >> r;
    const long long rem = M & ((1LL << r) - 1);
    const long long half = 1LL << (r - 1);
    q += (rem > half || (rem == half && (q & 1))) ? 1 : 0;
  }
  return (bits >> 63) ? -q : q;
}

}  // namespace tv
