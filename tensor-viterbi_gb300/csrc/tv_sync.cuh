// tv_sync.cuh -- cross-CTA messaging for the persistent grid decoder.
//
// Every wait is bounded: it gives up after `limit` SM clock cycles or when
// another CTA raised the abort word, and the caller then records an error
// status and returns.  No wait in this file can hang a GPU.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

namespace tv {

__device__ __forceinline__ unsigned ld_acquire_u32(const unsigned* p) {
  unsigned v;
  asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ int ld_relaxed_i32(const int* p) {
  int v;
  asm volatile("ld.relaxed.gpu.global.s32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ void st_release_u32(unsigned* p, unsigned v) {
  asm volatile("st.release.gpu.global.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}
__device__ __forceinline__ unsigned long long ld_relaxed_u64(const unsigned long long* p) {
  unsigned long long v;
  asm volatile("ld.relaxed.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ void st_relaxed_u64(unsigned long long* p, unsigned long long v) {
  asm volatile("st.relaxed.gpu.global.u64 [%0], %1;" ::"l"(p), "l"(v) : "memory");
}

// A message of three 64-bit words, each carrying the 32-bit step tag in its
// high half.  Single 8-byte stores are single-copy atomic, so a reader that
// sees the expected tag in all three words holds a consistent message
// without any fence: one L2 round trip per message.
constexpr int MSG_WORDS = 3;
struct TaggedMsg {
  unsigned long long w[MSG_WORDS];
};

__device__ __forceinline__ void msg_pack(TaggedMsg& m, unsigned tag, double v, int d, int i) {
  const unsigned long long bits = (unsigned long long)__double_as_longlong(v);
  const unsigned long long hi = (unsigned long long)tag << 32;
  m.w[0] = hi | (bits & 0xffffffffull);
  m.w[1] = hi | (bits >> 32);
  m.w[2] = hi | ((unsigned long long)(d & 0xffff) << 16) | (unsigned long long)(i & 0xffff);
}

__device__ __forceinline__ bool msg_tag_ok(const TaggedMsg& m, unsigned tag) {
  return (unsigned)(m.w[0] >> 32) == tag && (unsigned)(m.w[1] >> 32) == tag && (unsigned)(m.w[2] >> 32) == tag;
}

__device__ __forceinline__ void msg_unpack(const TaggedMsg& m, double& v, int& d, int& i) {
  const unsigned long long bits = (m.w[0] & 0xffffffffull) | ((m.w[1] & 0xffffffffull) << 32);
  v = __longlong_as_double((long long)bits);
  d = (int)((m.w[2] >> 16) & 0xffff);
  i = (int)(m.w[2] & 0xffff);
}

__device__ __forceinline__ void msg_store(unsigned long long* dst, const TaggedMsg& m) {
  st_relaxed_u64(dst + 0, m.w[0]);
  st_relaxed_u64(dst + 1, m.w[1]);
  st_relaxed_u64(dst + 2, m.w[2]);
}

__device__ __forceinline__ void msg_load(const unsigned long long* src, TaggedMsg& m) {
  m.w[0] = ld_relaxed_u64(src + 0);
  m.w[1] = ld_relaxed_u64(src + 1);
  m.w[2] = ld_relaxed_u64(src + 2);
}

// Poll until the message carries `tag`.  Returns false on abort / timeout.
__device__ __forceinline__ bool msg_wait(const unsigned long long* src, unsigned tag, TaggedMsg& m,
                                         const int* abort_flag, long long limit) {
  if (msg_tag_ok(m, tag)) return true;
  const long long t0 = clock64();
  for (;;) {
    msg_load(src, m);
    if (msg_tag_ok(m, tag)) return true;
    if (ld_relaxed_i32(abort_flag)) return false;
    if (clock64() - t0 > limit) return false;
    __nanosleep(20);
  }
}

// A 64-bit payload sent as two tagged words (low half, high half).
__device__ __forceinline__ void tagged64_store(unsigned long long* dst, unsigned tag, unsigned long long payload) {
  const unsigned long long hi = (unsigned long long)tag << 32;
  st_relaxed_u64(dst + 0, hi | (payload & 0xffffffffull));
  st_relaxed_u64(dst + 1, hi | (payload >> 32));
}

// Loads a tagged 64-bit payload, polling until both halves carry `tag`.
__device__ __forceinline__ bool tagged64_load(const unsigned long long* src, unsigned tag, unsigned long long& payload,
                                              const int* abort_flag, long long limit) {
  unsigned long long a = ld_relaxed_u64(src), b = ld_relaxed_u64(src + 1);
  if ((unsigned)(a >> 32) != tag || (unsigned)(b >> 32) != tag) {
    const long long t0 = clock64();
    for (;;) {
      __nanosleep(20);
      a = ld_relaxed_u64(src);
      b = ld_relaxed_u64(src + 1);
      if ((unsigned)(a >> 32) == tag && (unsigned)(b >> 32) == tag) break;
      if (ld_relaxed_i32(abort_flag)) return false;
      if (clock64() - t0 > limit) return false;
    }
  }
  payload = (a & 0xffffffffull) | ((b & 0xffffffffull) << 32);
  return true;
}

// Poll a monotonic counter until it reaches `target`.
__device__ __forceinline__ bool wait_geq(const unsigned* p, unsigned target, unsigned& seen, const int* abort_flag,
                                         long long limit) {
  seen = ld_acquire_u32(p);
  if (seen >= target) return true;
  const long long t0 = clock64();
  for (;;) {
    seen = ld_acquire_u32(p);
    if (seen >= target) return true;
    if (ld_relaxed_i32(abort_flag)) return false;
    if (clock64() - t0 > limit) return false;
    __nanosleep(20);
  }
}

}  // namespace tv
