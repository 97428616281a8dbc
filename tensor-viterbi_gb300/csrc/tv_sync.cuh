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

// A message of five 64-bit words, each carrying the 32-bit step tag in its
// high half: two 64-bit payloads in two halves each, and a 32-bit payload.
// Single 8-byte stores are single-copy atomic, so a reader that sees the
// expected tag in every word holds a consistent message without any fence:
// one L2 round trip per message.
constexpr int MSG_WORDS = 5;
struct TaggedMsg {
  unsigned long long w[MSG_WORDS];
};

__device__ __forceinline__ void msg_pack(TaggedMsg& m, unsigned tag, long long a, long long b, unsigned c) {
  const unsigned long long hi = (unsigned long long)tag << 32;
  m.w[0] = hi | ((unsigned long long)a & 0xffffffffull);
  m.w[1] = hi | ((unsigned long long)a >> 32);
  m.w[2] = hi | ((unsigned long long)b & 0xffffffffull);
  m.w[3] = hi | ((unsigned long long)b >> 32);
  m.w[4] = hi | c;
}

__device__ __forceinline__ bool msg_tag_ok(const TaggedMsg& m, unsigned tag) {
  bool ok = true;
#pragma unroll
  for (int k = 0; k < MSG_WORDS; ++k) ok = ok && (unsigned)(m.w[k] >> 32) == tag;
  return ok;
}

__device__ __forceinline__ void msg_unpack(const TaggedMsg& m, long long& a, long long& b, unsigned& c) {
  a = (long long)((m.w[0] & 0xffffffffull) | ((m.w[1] & 0xffffffffull) << 32));
  b = (long long)((m.w[2] & 0xffffffffull) | ((m.w[3] & 0xffffffffull) << 32));
  c = (unsigned)(m.w[4] & 0xffffffffull);
}

__device__ __forceinline__ void msg_store(unsigned long long* dst, const TaggedMsg& m) {
#pragma unroll
  for (int k = 0; k < MSG_WORDS; ++k) st_relaxed_u64(dst + k, m.w[k]);
}

__device__ __forceinline__ void msg_load(const unsigned long long* src, TaggedMsg& m) {
#pragma unroll
  for (int k = 0; k < MSG_WORDS; ++k) m.w[k] = ld_relaxed_u64(src + k);
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
