// tv_host.cu -- host side of the GB300 decoder and its C ABI (include/tv_gb300.h).
//
// Replaces the reference's host driver hsmm::decode_tensor_viterbi_cuda
// (src/hsmm.cu:604-720) and its pybind11 entry (src/bindings.cpp:104-114).
// Differences by design:
//   * the model is uploaded once (tv_model) instead of per call;
//   * back-pointers stay on the device and the backtrace runs there, so only
//     the T-int path and the log-likelihood cross to the host;
//   * errors come back as status codes instead of exit(EXIT_FAILURE)
//     (src/hsmm.cu:22-30).
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <mutex>
#include <set>
#include <utility>
#include <tuple>
#include <string>
#include <vector>

#include "../../include/tv_gb300.h"
#include "tv_cta.cuh"
#include "tv_grid.cuh"
#include "tv_floor.cuh"
#include "tv_fb.cuh"

namespace {

thread_local std::string g_err;

int fail(int code, const std::string& msg) {
  g_err = msg;
  return code;
}

#define TV_CUDA(call)                                                                   \
  do {                                                                                  \
    cudaError_t e_ = (call);                                                            \
    if (e_ != cudaSuccess)                                                              \
      return fail(TV_ECUDA, std::string(#call) + ": " + cudaGetErrorString(e_));       \
  } while (0)

// Stream-ordered allocation for the calling thread: while set (the decode
// server's scheduler sets it around each request), device buffers come from
// the device's memory pool in the order of that stream and are freed the same
// way, so finishing one request never waits for the others (cudaFree would
// synchronise the whole device).  Uploads into such buffers go on the same
// stream.
thread_local cudaStream_t g_alloc_stream = nullptr;
thread_local bool g_alloc_async = false;

template <class T>
struct DevBuf {
  T* p = nullptr;
  size_t n = 0;
  cudaStream_t st = nullptr;  // stream-ordered buffer: its stream
  bool async = false;
  DevBuf() = default;
  DevBuf(const DevBuf&) = delete;
  DevBuf& operator=(const DevBuf&) = delete;
  ~DevBuf() { release(); }
  int ensure(size_t count) {
    if (count <= n && p) return TV_OK;
    release();
    if (count == 0) count = 1;
    cudaError_t e;
    if (g_alloc_async) {
      e = cudaMallocAsync((void**)&p, count * sizeof(T), g_alloc_stream);
      st = g_alloc_stream;
      async = true;
    } else {
      e = cudaMalloc(&p, count * sizeof(T));
      if (e == cudaErrorMemoryAllocation) {
        // memory a stream-ordered pool keeps for reuse: give it back, retry once
        cudaGetLastError();
        int dev = 0;
        cudaMemPool_t pool;
        if (cudaGetDevice(&dev) == cudaSuccess && cudaDeviceGetDefaultMemPool(&pool, dev) == cudaSuccess) {
          cudaDeviceSynchronize();
          cudaMemPoolTrimTo(pool, 0);
          e = cudaMalloc(&p, count * sizeof(T));
        }
      }
      async = false;
    }
    if (e != cudaSuccess) {
      p = nullptr;
      cudaGetLastError();  // an allocation failure is not sticky; do not let it resurface later
      return fail(TV_ENOMEM, std::string("device allocation: ") + cudaGetErrorString(e));
    }
    n = count;
    return TV_OK;
  }
  void release() {
    if (p) {
      if (async) cudaFreeAsync(p, st);
      else cudaFree(p);
    }
    p = nullptr;
    n = 0;
  }
};

// Host-to-device upload on the thread's allocation stream when set.
cudaError_t upload(void* dst, const void* src, size_t bytes) {
  if (g_alloc_async) return cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice, g_alloc_stream);
  return cudaMemcpy(dst, src, bytes, cudaMemcpyHostToDevice);
}

constexpr int kThreads = 256;  // one-CTA kernel: single decodes, the server, the static path

// CTA shapes (threads per CTA) the batched decode chooses from.  The step
// loop gives each warp whole states, so the best shape depends on N (warps
// per state round), on D (the lanes' share of a state's window) and on how
// many CTAs the window's shared memory lets an SM hold.
constexpr int kCtaShapes[] = {128, 256, 384, 512};
using CtaKernelFn = void (*)(tv::ModelView, tv::BatchView, tv::CtaLayout, unsigned char*);
CtaKernelFn cta_kernel_for(int threads) {
  switch (threads) {
    case 128: return tv::cta_decode_kernel<128>;
    case 384: return tv::cta_decode_kernel<384>;
    case 512: return tv::cta_decode_kernel<512>;
    default: return tv::cta_decode_kernel<256>;
  }
}

// Dynamic shared-memory limits.  A kernel that takes dynamic shared memory
// gets the device's whole opt-in limit, less its own static shared memory,
// once per device before its first launch there, and never a smaller value
// afterwards.  The limit is process-wide state of the kernel: a value set per
// call could be overwritten by another thread between its set and its launch,
// and a launch needing more than the last value set would fail.
std::mutex g_smem_mu;
std::set<std::pair<int, const void*>> g_smem_done;

int raise_smem_limit(const void* kern) {
  int dev = 0;
  TV_CUDA(cudaGetDevice(&dev));
  std::lock_guard<std::mutex> lk(g_smem_mu);
  if (g_smem_done.count({dev, kern})) return TV_OK;
  int optin = 0;
  TV_CUDA(cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev));
  cudaFuncAttributes fa{};
  TV_CUDA(cudaFuncGetAttributes(&fa, kern));
  TV_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, optin - (int)fa.sharedSizeBytes));
  g_smem_done.insert({dev, kern});
  return TV_OK;
}

// Autotuned CTA shape per (N, D, window in shared memory), measured once per
// process on the first large batch of that shape.
std::mutex g_tune_mu;
std::map<std::tuple<int, int, int>, int> g_tuned;

// Log-space survival, accumulated from d = D-1 downwards with the running
// two-term log-sum-exp of the reference (src/hsmm.cu:79-99); computed on the
// host so it uses the same libm as the reference's CPU path.  Output [j][d].
void survival_T(int N, int D, const double* dur, std::vector<double>& survT) {
  survT.assign((size_t)N * D, 0.0);
  const double ninf = -INFINITY;
  for (int j = 0; j < N; ++j) {
    double acc = ninf;
    for (int d = D - 1; d >= 0; --d) {
      const double lp = dur[(size_t)d * N + j];
      const double hi = (acc < lp) ? lp : acc;
      acc = (hi == ninf) ? lp : hi + std::log(std::exp(acc - hi) + std::exp(lp - hi));
      survT[(size_t)j * D + d] = acc;
    }
  }
}

bool all_finite(const double* x, size_t n, double* maxabs) {
  double m = 0.0;
  for (size_t k = 0; k < n; ++k) {
    if (!std::isfinite(x[k])) return false;
    m = std::max(m, std::fabs(x[k]));
  }
  *maxabs = m;
  return true;
}

__global__ void quantize_kernel(const double* __restrict__ src, long long* __restrict__ dst, size_t n, double scale) {
  for (size_t k = blockIdx.x * (size_t)blockDim.x + threadIdx.x; k < n; k += (size_t)gridDim.x * blockDim.x)
    dst[k] = __double2ll_rn(src[k] * scale);
}

}  // namespace

struct tv_model_s {
  int N = 0, O = 0, D = 0;
  double emax = 0, tmax = 0, dmax = 0, smax = 0;
  DevBuf<double> em, trans, start, durT, survT;
  DevBuf<long long> qem, qtr, qdurT;
  int qf = -1;  // fraction bits the quantised tables were built for
  // per-decode scratch
  DevBuf<uint32_t> psi;
  DevBuf<int> status;
  DevBuf<int> counter;
  DevBuf<int64_t> off;
  DevBuf<int> order;
  DevBuf<int64_t> tune_off;
  DevBuf<unsigned char> scratch;
  int batch_threads = 0;  // CTA shape of the last batched launch
  int batch_grid = 0;     // and its number of CTAs
  DevBuf<int32_t> obs_tmp, path_tmp;
  DevBuf<double> ll_tmp;
  int64_t last_launches = 0;
  int sm_count = 0;
  // grid-kernel scratch (single long sequences)
  DevBuf<unsigned long long> msgs;  // slot messages, partial messages, exact delta ring
  DevBuf<double> dinit, ck, hwin;
  DevBuf<long long> wrange;
  DevBuf<unsigned char> wglob;  // worker windows in global memory (large N*D)
  DevBuf<int> seg_first, seg_count, seg_base, gflags;
  int plan_key_N = -1, plan_key_D = -1, plan_key_G = -1, plan_key_L2 = -1;
  tv::GridParams plan{};
  int path_pref = TV_PATH_AUTO, grid_ctas = 0, last_path = 0;
  // test-only: a worker partial message the next grid decode drops
  unsigned drop_tag = 0;
  int drop_seg = -1;
  // optional events around the main kernel
  bool timing = false, timed = false;
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
  std::mutex mu;
};

namespace {

struct Quant {
  int f;
  double scale;
  long long margin;
};

// Fixed-point format and certified margin for a decode of length up to T.
// Every candidate score V = (E + delta) + (tr + dur) is approximated by the
// fixed-point sum of quantised terms; its error is bounded by
//   (D+1) q/2      emission prefix: D+1 rounded terms
// + D^2 u emax     the reference's own rounding of the window fold
// + 3 q/2          quantised delta, transition, duration
// + 3 u S          rounding inside V, S bounding every partial sum
// (u = 2^-53, q = 2^-f).  Two candidates whose fixed-point scores differ by
// more than twice that bound compare the same way exactly.
Quant choose_quant(const tv_model_s* m, int64_t T) {
  const double u = std::ldexp(1.0, -53);
  const double per = m->emax + m->tmax + m->dmax;
  const double S = (double)T * per + m->smax + (double)m->D * m->emax + m->tmax + m->dmax + 1.0;
  const double Vb = 2.0 * (S + (double)T * m->emax) + 16.0;
  int f = (int)std::floor(61.0 - std::log2(Vb));
  f = std::max(0, std::min(40, f));
  const double q = std::ldexp(1.0, -f);
  const double err = ((double)m->D + 1.0) * q * 0.5 + (double)m->D * (double)m->D * u * m->emax + 1.5 * q + 3.0 * u * S;
  Quant Q;
  Q.f = f;
  Q.scale = std::ldexp(1.0, f);
  Q.margin = (long long)std::ceil(2.0 * err * Q.scale) + 8;
  return Q;
}

void mark_start(tv_model_s* m, cudaStream_t st) {
  m->timed = false;
  if (m->timing && m->ev0) cudaEventRecord(m->ev0, st);
}

void mark_end(tv_model_s* m, cudaStream_t st) {
  if (m->timing && m->ev1 && cudaEventRecord(m->ev1, st) == cudaSuccess) m->timed = true;
}

int prepare_quant(tv_model_s* m, const Quant& Q, cudaStream_t st) {
  if (m->qf == Q.f) return TV_OK;
  int rc;
  if ((rc = m->qem.ensure((size_t)m->O * m->N)) != TV_OK) return rc;
  if ((rc = m->qtr.ensure((size_t)m->N * m->N)) != TV_OK) return rc;
  if ((rc = m->qdurT.ensure((size_t)m->N * m->D)) != TV_OK) return rc;
  quantize_kernel<<<64, 256, 0, st>>>(m->em.p, m->qem.p, (size_t)m->O * m->N, Q.scale);
  quantize_kernel<<<64, 256, 0, st>>>(m->trans.p, m->qtr.p, (size_t)m->N * m->N, Q.scale);
  quantize_kernel<<<64, 256, 0, st>>>(m->durT.p, m->qdurT.p, (size_t)m->N * m->D, Q.scale);
  TV_CUDA(cudaGetLastError());
  m->last_launches += 3;
  m->qf = Q.f;
  return TV_OK;
}

tv::ModelView view(const tv_model_s* m, const Quant& Q) {
  tv::ModelView v{};
  v.N = m->N; v.O = m->O; v.D = m->D;
  v.em = m->em.p; v.trans = m->trans.p; v.start = m->start.p;
  v.durT = m->durT.p; v.survT = m->survT.p;
  v.qem = m->qem.p; v.qtr = m->qtr.p; v.qdurT = m->qdurT.p;
  v.scale = Q.scale;
  v.margin = Q.margin;
  return v;
}

int check_obs_host(const int32_t* obs, int64_t T, int O) {
  for (int64_t t = 0; t < T; ++t)
    if (obs[t] < 0 || obs[t] >= O)
      return fail(TV_ERANGE, "observation " + std::to_string(obs[t]) + " at t=" + std::to_string(t) +
                                 " outside [0, " + std::to_string(O) + ")");
  return TV_OK;
}

// Launches the CTA-per-sequence kernel over n_seq sequences whose
// observations / paths live on the device.  `off_host` has n_seq+1 entries.
int launch_batch(tv_model_s* m, int n_seq, const int64_t* off_host, const int32_t* obs_dev,
                 int32_t* path_dev, double* ll_dev, cudaStream_t st, bool tune = false) {
  const int N = m->N, D = m->D;
  int64_t Tmax = 0;
  for (int k = 0; k < n_seq; ++k) {
    const int64_t T = off_host[k + 1] - off_host[k];
    if (T <= 0) return fail(TV_EINVAL, "empty sequence " + std::to_string(k));
    if (T < D) return fail(TV_ESHORT, "sequence " + std::to_string(k) + " has T=" + std::to_string(T) +
                                          " < D=" + std::to_string(D) + "; the reference initialisation needs T >= D");
    Tmax = std::max(Tmax, T);
  }
  const Quant Q = choose_quant(m, Tmax);
  int rc;
  if ((rc = prepare_quant(m, Q, st)) != TV_OK) return rc;

  const int64_t total = off_host[n_seq];
  if ((rc = m->psi.ensure((size_t)total * N)) != TV_OK) return rc;
  if ((rc = m->status.ensure((size_t)n_seq)) != TV_OK) return rc;
  if ((rc = m->counter.ensure(1)) != TV_OK) return rc;
  if ((rc = m->off.ensure((size_t)n_seq + 1)) != TV_OK) return rc;
  TV_CUDA(cudaMemcpyAsync(m->off.p, off_host, sizeof(int64_t) * (n_seq + 1), cudaMemcpyHostToDevice, st));
  TV_CUDA(cudaMemsetAsync(m->counter.p, 0, sizeof(int), st));
  // Longest sequences first: the persistent CTAs then finish close together.
  const int* order_dev = nullptr;
  if (n_seq > 1) {
    std::vector<int> ord((size_t)n_seq);
    for (int k = 0; k < n_seq; ++k) ord[k] = k;
    std::stable_sort(ord.begin(), ord.end(), [&](int a, int b) {
      return off_host[a + 1] - off_host[a] > off_host[b + 1] - off_host[b];
    });
    if ((rc = m->order.ensure((size_t)n_seq)) != TV_OK) return rc;
    // pageable source: the copy is staged before the call returns
    TV_CUDA(cudaMemcpyAsync(m->order.p, ord.data(), sizeof(int) * n_seq, cudaMemcpyHostToDevice, st));
    order_dev = m->order.p;
  }

  int dev = 0;
  TV_CUDA(cudaGetDevice(&dev));
  int smem_optin = 0;
  TV_CUDA(cudaDeviceGetAttribute(&smem_optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev));
  const size_t static_smem = 64;
  // Work area in shared memory when it fits; then, per CTA shape, the
  // duration table stays in global memory when that lets more CTAs share an
  // SM (the window scan is bound by the SM's FP64 unit and the phases'
  // barriers, which more resident CTAs overlap).
  const tv::CtaLayout L_full = tv::make_cta_layout(N, D), L_lean = tv::make_cta_layout(N, D, true);
  tv::CtaLayout L = L_full;
  size_t dyn = 0;
  if (L.bytes + static_smem <= (size_t)smem_optin) {
    L.in_smem = 1;
    dyn = L.bytes;
  }
  // grid of a shape: as many CTAs as the SMs hold, at most one per sequence
  auto prepare = [&](int threads, int n, int& grid) -> int {
    const CtaKernelFn kern = cta_kernel_for(threads);
    if (L_full.bytes + static_smem <= (size_t)smem_optin) {
      const int rc2 = raise_smem_limit((const void*)kern);
      if (rc2 != TV_OK) return rc2;
      int pf = 1, pl = 1;
      TV_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&pf, kern, threads, L_full.bytes));
      TV_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&pl, kern, threads, L_lean.bytes));
      // only when the batch has more sequences than the full layout's CTAs
      // can hold (a lone CTA is faster with the table in shared memory)
      L = (pl > pf && n > m->sm_count * pf) ? L_lean : L_full;
      L.in_smem = 1;
      dyn = L.bytes;
    }
    int per_sm = 1;
    TV_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, threads, dyn));
    grid = std::max(1, std::min(n, m->sm_count * std::max(per_sm, 1)));
    if (!L.in_smem) {
      int rc2;
      if ((rc2 = m->scratch.ensure((size_t)grid * L.bytes)) != TV_OK) return rc2;
    }
    return TV_OK;
  };
  tv::BatchView bv{};
  bv.obs = obs_dev;
  bv.off = m->off.p;
  bv.path = path_dev;
  bv.loglik = ll_dev;
  bv.psi = m->psi.p;
  bv.status = m->status.p;
  bv.next = m->counter.p;
  bv.order = order_dev;
  bv.n_seq = n_seq;

  // The CTA shape: the tuned one for this (N, D, placement), else 256.  A
  // batch of at least two waves of CTAs with no tuned shape yet measures
  // every shape and keeps the one with the highest rate; TV_AUTOTUNE=0 turns
  // this off.  Each shape runs one wave of its own grid (the CTAs that share
  // an SM differ between shapes) on sequences of 8 D steps cut from the
  // batch's observations (mostly the steady state of the recurrence, not the
  // initialisation), and is scored by steps per second.
  int threads = kThreads;
  const auto key = std::make_tuple(N, D, L.in_smem);
  bool tuned = false;
  if (tune) {
    std::lock_guard<std::mutex> lk(g_tune_mu);
    auto it = g_tuned.find(key);
    if (it != g_tuned.end()) {
      threads = it->second;
      tuned = true;
    }
  }
  const char* env = std::getenv("TV_AUTOTUNE");
  const bool tune_on = !(env && env[0] == '0');
  int64_t trial_len = 8LL * D;  // shorter (down to 2 D) when the batch holds fewer than 4 waves of them
  if (total / trial_len < 4LL * m->sm_count) trial_len = std::max<int64_t>(2LL * D, total / (4LL * m->sm_count));
  if (!tuned && tune_on && tune && n_seq >= 2 * m->sm_count && total / trial_len >= 2LL * m->sm_count) {
    struct Events {  // released on every return path
      cudaEvent_t a = nullptr, b = nullptr;
      ~Events() {
        if (a) cudaEventDestroy(a);
        if (b) cudaEventDestroy(b);
      }
    } ev;
    TV_CUDA(cudaEventCreate(&ev.a));
    TV_CUDA(cudaEventCreate(&ev.b));
    cudaEvent_t e0 = ev.a, e1 = ev.b;
    const int max_trials = (int)std::min<int64_t>(n_seq, total / trial_len);
    if ((rc = m->tune_off.ensure((size_t)max_trials + 1)) != TV_OK) return rc;
    std::vector<int64_t> toff((size_t)max_trials + 1);
    for (int k = 0; k <= max_trials; ++k) toff[k] = (int64_t)k * trial_len;
    // pageable source: the copy is staged before the call returns
    TV_CUDA(cudaMemcpyAsync(m->tune_off.p, toff.data(), sizeof(int64_t) * toff.size(), cudaMemcpyHostToDevice,
                            st));
    double best_rate = 0.0;
    int best = kThreads;
    for (int shape : kCtaShapes) {
      int grid = 1;
      if ((rc = prepare(shape, max_trials, grid)) != TV_OK) break;
      tv::BatchView sv = bv;
      sv.off = m->tune_off.p;
      sv.order = nullptr;
      sv.n_seq = grid;  // one full wave
      TV_CUDA(cudaMemsetAsync(m->counter.p, 0, sizeof(int), st));
      TV_CUDA(cudaEventRecord(e0, st));
      cta_kernel_for(shape)<<<grid, shape, dyn, st>>>(view(m, Q), sv, L, L.in_smem ? nullptr : m->scratch.p);
      TV_CUDA(cudaGetLastError());
      TV_CUDA(cudaEventRecord(e1, st));
      TV_CUDA(cudaEventSynchronize(e1));
      float ms = 0.0f;
      TV_CUDA(cudaEventElapsedTime(&ms, e0, e1));
      m->last_launches += 1;
      const double rate = (double)grid * (double)trial_len / std::max(1e-6, (double)ms);
      if (rate > best_rate) {
        best_rate = rate;
        best = shape;
      }
    }
    if (rc != TV_OK) return rc;
    threads = best;
    std::lock_guard<std::mutex> lk(g_tune_mu);
    g_tuned[key] = best;
    TV_CUDA(cudaMemsetAsync(m->counter.p, 0, sizeof(int), st));
  }
  int grid = 1;
  if ((rc = prepare(threads, n_seq, grid)) != TV_OK) return rc;
  m->batch_threads = threads;
  m->batch_grid = grid;
  mark_start(m, st);
  cta_kernel_for(threads)<<<grid, threads, dyn, st>>>(view(m, Q), bv, L, L.in_smem ? nullptr : m->scratch.p);
  TV_CUDA(cudaGetLastError());
  mark_end(m, st);
  m->last_launches += 1;
  return TV_OK;
}


// Assigns the N*D window cells (state-major, ring slot minor) to the worker
// CTAs.  When every state can get k >= 1 whole workers, each state's ring is
// cut into k equal parts (one segment per worker, all tables of a worker in
// its shared memory); otherwise the cells are cut into equal contiguous
// chunks that may span several states.  A worker's intersection with a
// state's row is a segment and yields one partial winner per step.
bool plan_grid_nd(int N, int D, int G, int smem_optin, bool force_l2, tv::GridParams& P, std::vector<long long>& wr,
                  std::vector<int>& first, std::vector<int>& count, std::vector<int>& base) {
  const int L = tv::GRID_L;
  if (G < 2 || D <= L || N > tv::GRID_MAX_N || D > 65535) return false;
  const int Gw = G - 1;
  const long long ND = (long long)N * D;
  long long chunk = 0;
  int S = 0, max_seg = 0;
  long long seg_cost = 0;  // cost of a worker's extra segment, in cells (0: equal chunks)
  auto partition = [&](bool row_aligned) {
    wr.assign(2 * (size_t)Gw, 0);
    const int k = Gw / N;
    if (row_aligned && k >= 1) {
      const int parts = (int)std::min<long long>(k, D);
      const long long part = (D + parts - 1) / parts;
      int w = 0;
      for (int j = 0; j < N; ++j)
        for (int q = 0; q < parts; ++q, ++w) {
          const long long lo = (long long)j * D + (long long)q * part;
          const long long hi = std::min((long long)j * D + (long long)(q + 1) * part, (long long)(j + 1) * D);
          wr[2 * w] = lo;
          wr[2 * w + 1] = std::max(lo, hi);
        }
      for (; w < Gw; ++w) wr[2 * w] = wr[2 * w + 1] = ND;
      chunk = part;
    } else if (seg_cost <= 0) {
      chunk = (ND + Gw - 1) / Gw;
      for (int w = 0; w < Gw; ++w) {
        const long long lo = std::min((long long)w * chunk, ND), hi = std::min(lo + chunk, ND);
        wr[2 * w] = lo;
        wr[2 * w + 1] = hi;
      }
    } else {
      // Contiguous chunks of equal cost, a cell costing 1 and every segment
      // after a worker's first costing seg_cost more (a second state's loop
      // and reduction): the smallest per-worker cost C whose greedy cover
      // needs at most Gw workers.
      auto cover = [&](long long C, bool fill) -> int {
        long long p = 0;
        int w = 0;
        while (p < ND) {
          if (w == Gw) return Gw + 1;
          const long long lo = p;
          long long b = C;
          for (;;) {
            const long long end = (p / D + 1) * D;  // end of this state's row
            const long long take = std::min(b, end - p);
            p += take;
            b -= take;
            if (p == ND || p < end || b <= seg_cost) break;
            b -= seg_cost;  // continue into the next state
          }
          if (fill) {
            wr[2 * w] = lo;
            wr[2 * w + 1] = p;
          }
          ++w;
        }
        if (fill)
          for (int v = w; v < Gw; ++v) wr[2 * v] = wr[2 * v + 1] = ND;
        return w;
      };
      long long lo = (ND + Gw - 1) / Gw, hi = ND;
      while (lo < hi) {
        const long long mid = (lo + hi) / 2;
        if (cover(mid, false) <= Gw) hi = mid;
        else lo = mid + 1;
      }
      cover(lo, true);
      chunk = 0;
      for (int w = 0; w < Gw; ++w) chunk = std::max(chunk, wr[2 * w + 1] - wr[2 * w]);
    }
    first.assign(N, 0);
    count.assign(N, 0);
    base.assign(Gw, 0);
    std::vector<int> seen(N, 0);
    S = 0;
    max_seg = 0;
    for (int w = 0; w < Gw; ++w) {
      const long long lo = wr[2 * w], hi = wr[2 * w + 1];
      base[w] = S;
      if (lo >= hi) continue;
      const int ja = (int)(lo / D), jb = (int)((hi - 1) / D);
      for (int j = ja; j <= jb; ++j) {
        if (!seen[j]) { seen[j] = 1; first[j] = S; }
        count[j]++;
        S++;
      }
      max_seg = std::max(max_seg, jb - ja + 1);
    }
  };
  // Head roles: the critical lanes and two state-helper groups, a lane per
  // state each, and intake lanes that take two segments each and cover the
  // states.
  auto round32 = [](int x) { return (x + 31) / 32 * 32; };
  auto intake_threads = [&](int S_) { return round32(std::max((S_ + 1) / 2, N)); };
  auto head_roles_fit = [&](int S_) { return 3 * round32(N) + intake_threads(S_) <= tv::GRID_THREADS; };
  // Cells are split per state (row-aligned) when every state gets whole
  // workers, so that a worker's duration and transition rows are one state's;
  // otherwise in equal contiguous chunks that may span states.
  partition(true);
  // Window in shared memory when a worker's share fits there: the duration
  // rows (8 B fixed point + 8 B exact per d) and transition rows of its
  // states, and per cell the slot score, selected delta, three window-sum
  // buffers (8 B each) and the argmax word (2 B); the scan's per-warp
  // results for two steps.
  auto red_bytes = [&](int nw) {
    return (unsigned long long)std::max(2 * max_seg * nw * sizeof(tv::Top2), 32 * sizeof(tv::ExactBest));
  };
  auto smem_window_bytes = [&]() {
    unsigned long long o = 0;
    o = tv::tv_align(o + (unsigned long long)max_seg * D * 8);
    o = tv::tv_align(o + (unsigned long long)max_seg * D * 8);
    o = tv::tv_align(o + (unsigned long long)max_seg * N * 8);
    for (int a = 0; a < 5; ++a) o = tv::tv_align(o + (unsigned long long)chunk * 8);
    o = tv::tv_align(o + (unsigned long long)chunk * 2);
    o = tv::tv_align(o + red_bytes(tv::WORKER_THREADS / 32));
    o = tv::tv_align(o + (unsigned long long)2 * max_seg * 8);
    return o;
  };
  const bool global_window = force_l2 || smem_window_bytes() + 256 > (unsigned long long)smem_optin;
  if (global_window) {
    // In global memory the tables come from the model, so equal contiguous
    // chunks over all workers balance the scan best, as long as the head's
    // intake roles (one lane per segment) still fit.
    std::vector<long long> wr0 = wr;
    std::vector<int> f0 = first, c0 = count, b0 = base;
    const long long chunk0 = chunk;
    const int S0 = S, ms0 = max_seg;
    // With the window in L2 a worker's second segment costs about a third of
    // an equal share of the scan (its own loop start and reduction, measured
    // at N=100 D=1e4), so such workers get fewer cells.
    seg_cost = (ND + Gw - 1) / Gw / 3;
    partition(false);
    if (!head_roles_fit(S) || max_seg > 32) {
      wr = wr0; first = f0; count = c0; base = b0; chunk = chunk0; S = S0; max_seg = ms0;
    }
  }
  if (S > tv::GRID_THREADS || max_seg > 32 || !head_roles_fit(S)) return false;
  P = tv::GridParams{};
  P.G = G; P.L = L; P.S = S; P.Rd = D + 2 * L + 8;
  P.M = (D + tv::CK_STRIDE - 1) / tv::CK_STRIDE;
  P.chunk = chunk; P.max_seg = max_seg;
  unsigned long long o = 0;
  if (!global_window) {
    P.w_qd = o;   o = tv::tv_align(o + (unsigned long long)max_seg * D * 8);
    P.w_dur = o;  o = tv::tv_align(o + (unsigned long long)max_seg * D * 8);
    P.w_tr = o;   o = tv::tv_align(o + (unsigned long long)max_seg * N * 8);
    P.w_ctil = o; o = tv::tv_align(o + (unsigned long long)chunk * 8);
    P.w_dsel = o; o = tv::tv_align(o + (unsigned long long)chunk * 8);
    P.w_accs = tv::tv_align((unsigned long long)chunk * 8);
    P.w_acc = o;  o += 3 * P.w_accs;
    P.w_itil = o; o = tv::tv_align(o + (unsigned long long)chunk * 2);
    P.w_red = o;  o = tv::tv_align(o + red_bytes(tv::WORKER_THREADS / 32));
    P.w_emw = o;  o = tv::tv_align(o + (unsigned long long)2 * max_seg * 8);
    P.w_bytes = o;
  } else {
    // Each worker keeps its window in its own global-memory buffer (served by
    // L1/L2) and reads the duration and transition rows from the model.
    P.w_global = 1;
    unsigned long long g = 0;
    P.w_ctil = g; g = tv::tv_align(g + (unsigned long long)chunk * 8);
    P.w_dsel = g; g = tv::tv_align(g + (unsigned long long)chunk * 8);
    P.w_accs = tv::tv_align((unsigned long long)chunk * 8);
    P.w_acc = g;  g += 3 * P.w_accs;
    P.w_itil = g; g = tv::tv_align(g + (unsigned long long)chunk * 2);
    P.w_gstride = (g + 255) / 256 * 256;
    P.w_qd = P.w_dur = P.w_tr = 0;
    // The fixed-point duration rows, read every step by the scan, join shared
    // memory when they fit.
    const unsigned long long qbytes = tv::tv_align((unsigned long long)max_seg * D * 8);
    if (qbytes + red_bytes(tv::WORKER_THREADS_GW / 32) + 2 * (unsigned long long)max_seg * 8 + 512 <=
        (unsigned long long)smem_optin) {
      P.w_qd_smem = 1;
      P.w_qd = 0;
      o = qbytes;
    }
    P.w_red = o;  o = tv::tv_align(o + red_bytes(tv::WORKER_THREADS_GW / 32));
    P.w_emw = o;  o = tv::tv_align(o + (unsigned long long)2 * max_seg * 8);
    P.w_bytes = o;
  }
  o = 0;
  const int Np = (N + 15) / 16 * 16;
  P.Np = Np;
  P.cs_threads = round32(N);
  P.st_threads = round32(N);
  P.in_threads = intake_threads(S);
  // a second warp per 32 states for the upper half of the matvec, when the
  // block has room for it (at most 4 pairs: named barriers 10..13)
  P.cs_split = (4 * round32(N) + P.in_threads <= tv::GRID_THREADS && round32(N) <= 128) ? 1 : 0;
  P.block = std::max(P.cs_threads * (1 + P.cs_split) + 2 * P.st_threads + P.in_threads,
                     (P.w_global ? tv::WORKER_THREADS_GW : tv::WORKER_THREADS) + tv::WORKER_SERVICE);
  if (P.block > tv::GRID_THREADS) return false;
  P.h_xch = o;    o = tv::tv_align(o + (unsigned long long)N * 8);
  P.h_qcp = o;    o = tv::tv_align(o + (unsigned long long)N * (Np + 4) * 4);  // row stride Np + 4
  P.h_dqcp = o;   o = tv::tv_align(o + (unsigned long long)2 * Np * 4);
  P.h_dq = o;     o = tv::tv_align(o + (unsigned long long)2 * N * 8);
  P.h_ptil = o;   o = tv::tv_align(o + (unsigned long long)4 * N * 8);
  P.h_base = o;   o = tv::tv_align(o + 16);
  P.h_dstar = o;  o = tv::tv_align(o + (unsigned long long)(L + 1) * N * 8);
  P.h_ctil = o;   o = tv::tv_align(o + (unsigned long long)L * N * 8);
  P.h_itil = o;   o = tv::tv_align(o + (unsigned long long)L * N * 2);
  P.h_hwr = o;    o = tv::tv_align(o + (unsigned long long)tv::HWR * L * N * 8);
  P.h_qd = o;     o = tv::tv_align(o + (unsigned long long)N * L * 8);
  P.h_dur = o;    o = tv::tv_align(o + (unsigned long long)N * L * 8);
  P.h_prek = o;   o = tv::tv_align(o + (unsigned long long)2 * N * 8);
  P.h_pred = o;   o = tv::tv_align(o + (unsigned long long)2 * N * 4);
  P.h_prei = o;   o = tv::tv_align(o + (unsigned long long)2 * N * 4);
  P.h_prew = o;   o = tv::tv_align(o + (unsigned long long)2 * N * 8);
  P.h_preq = o;   o = tv::tv_align(o + (unsigned long long)2 * N * 8);
  P.h_pwq = o;    o = tv::tv_align(o + (unsigned long long)2 * S * 8);
  P.h_pwk = o;    o = tv::tv_align(o + (unsigned long long)2 * S * 8);
  P.h_pwd = o;    o = tv::tv_align(o + (unsigned long long)2 * S * 4);
  P.h_pwi = o;    o = tv::tv_align(o + (unsigned long long)2 * S * 4);
  P.h_psirec = o; o = tv::tv_align(o + (unsigned long long)4 * N * 4);
  P.h_tail = o;   o = tv::tv_align(o + (unsigned long long)N * 8);
  // The exact transition matrix and its fixed-point copy join the head's
  // shared memory when they fit; the exact one first (the fixed-point copy
  // is then computed from it: a multiply and a conversion).
  const unsigned long long nn8 = tv::tv_align((unsigned long long)N * N * 8);
  P.h_trh = o;
  P.trans_smem = o + nn8 + 256 <= (unsigned long long)smem_optin ? 1 : 0;
  if (P.trans_smem) o += nn8;
  P.h_qtr = o;
  P.qtr_smem = o + nn8 + 256 <= (unsigned long long)smem_optin ? 1 : 0;
  if (P.qtr_smem) o += nn8;
  P.h_bytes = o;
  P.timeout = 1LL << 31;  // SM clock cycles, about a second: no legitimate wait comes close
  P.copy_timeout = 1LL << 31;
  P.drop_tag = 0;
  P.drop_seg = -1;
  return std::max(P.w_bytes, P.h_bytes) + 256 <= (unsigned long long)smem_optin;
}

bool plan_grid(tv_model_s* m, int G, int smem_optin, bool force_l2, tv::GridParams& P, std::vector<long long>& wr,
               std::vector<int>& first, std::vector<int>& count, std::vector<int>& base) {
  return plan_grid_nd(m->N, m->D, G, smem_optin, force_l2, P, wr, first, count, base);
}

// The grid kernel instance for a plan: window in shared or global memory.
const void* grid_kernel_for(const tv::GridParams& P) {
  return P.w_global ? (const void*)tv::grid_decode_kernel<true> : (const void*)tv::grid_decode_kernel<false>;
}

int launch_grid(tv_model_s* m, const int32_t* obs_dev, int64_t T, int32_t* path_dev, double* ll_dev,
                cudaStream_t st, const tv::GridParams& P) {
  const int N = m->N, D = m->D;
  const Quant Q = choose_quant(m, T);
  if (Q.f < tv::COARSE_F) return fail(TV_ETOOBIG, "sequence too long for the grid kernel's fixed-point range");
  int rc;
  if ((rc = prepare_quant(m, Q, st)) != TV_OK) return rc;
  if ((rc = m->psi.ensure((size_t)T * N)) != TV_OK) return rc;
  const size_t slot_words = (size_t)tv::SLOT_RING * N * tv::SLOT_WORDS;
  const size_t part_words = (size_t)tv::PART_RING * P.S * tv::MSG_WORDS;
  const size_t dstar_words = (size_t)P.Rd * N * 2;
  if ((rc = m->msgs.ensure(slot_words + part_words + dstar_words)) != TV_OK) return rc;
  if ((rc = m->dinit.ensure((size_t)D * N)) != TV_OK) return rc;
  const int tmax = (int)std::min<int64_t>(D, T - 1);
  if ((rc = m->ck.ensure((size_t)std::max(tmax, 1) * P.M * N)) != TV_OK) return rc;
  if ((rc = m->hwin.ensure((size_t)T * tv::GRID_L * N)) != TV_OK) return rc;
  if ((rc = m->gflags.ensure(4)) != TV_OK) return rc;
  // Tags start at 1: a cleared buffer holds no valid message.
  TV_CUDA(cudaMemsetAsync(m->msgs.p, 0, sizeof(unsigned long long) * (slot_words + part_words + dstar_words), st));
  TV_CUDA(cudaMemsetAsync(m->gflags.p, 0, sizeof(int) * 4, st));
  tv::ModelView mv = view(m, Q);
  int* gabort = m->gflags.p + 1;
  int* gstatus = m->gflags.p + 2;
  tv::grid_check_obs<<<64, 256, 0, st>>>(obs_dev, T, m->O, gabort, gstatus);
  tv::grid_prep_init<<<(N + 127) / 128, 128, 0, st>>>(mv, obs_dev, m->dinit.p, gabort);
  m->last_launches += 2;
  if (tmax >= 1) {
    const long long nthr = (long long)tmax * N;
    tv::grid_prep_ck<<<(unsigned)((nthr + 255) / 256), 256, 0, st>>>(mv, obs_dev, m->ck.p, P.M, tmax, gabort);
    m->last_launches += 1;
  }
  {
    const long long nthr = T * N;
    tv::grid_prep_hwin<<<(unsigned)((nthr + 255) / 256), 256, 0, st>>>(mv, obs_dev, T, m->hwin.p, gabort);
    m->last_launches += 1;
  }
  TV_CUDA(cudaGetLastError());
  tv::GridBufs B{};
  B.obs = obs_dev;
  B.T = T;
  B.psi = m->psi.p;
  B.path = path_dev;
  B.loglik = ll_dev;
  B.slot_msg = m->msgs.p;
  B.part = m->msgs.p + slot_words;
  B.dstar = m->msgs.p + slot_words + part_words;
  B.dinit = m->dinit.p;
  B.ck = m->ck.p;
  B.hwin = m->hwin.p;
  B.wrange = m->wrange.p;
  if (P.w_global) {
    if ((rc = m->wglob.ensure((size_t)(P.G - 1) * P.w_gstride)) != TV_OK) return rc;
    B.wglob = m->wglob.p;
  }
  B.seg_first = m->seg_first.p;
  B.seg_count = m->seg_count.p;
  B.seg_base = m->seg_base.p;
  B.abort_flag = gabort;
  B.status = gstatus;
  B.site = m->gflags.p + 0;
  tv::GridParams Pc = P;
  // Packed coarse matvec: coarse unit 2^-COARSE_F.  Each coarse score is off
  // by < 2 units (two floors) from the fine one, which is within q + 3uS of
  // the exact value; a coarse runner-up gap above the margin certifies the
  // argmax over i.
  Pc.coarse_shift = Q.f - tv::COARSE_F;
  Pc.qf = Q.f;
  {
    const double u = std::ldexp(1.0, -53), q = std::ldexp(1.0, -Q.f), qc = std::ldexp(1.0, -tv::COARSE_F);
    const double S_ = (double)T * (m->emax + m->tmax + m->dmax) + m->smax + (double)m->D * m->emax + m->tmax + m->dmax;
    Pc.coarse_margin = 4 + (int)std::ceil(2.0 * (q + 3.0 * u * S_) / qc) + 2;
  }
  Pc.drop_tag = m->drop_tag;  // one decode only
  Pc.drop_seg = m->drop_seg;
  m->drop_tag = 0;
  m->drop_seg = -1;
  void* args[] = {&mv, &Pc, &B};
  const size_t dyn = std::max(P.w_bytes, P.h_bytes);
  const void* kern = grid_kernel_for(P);
  if ((rc = raise_smem_limit(kern)) != TV_OK) return rc;
  mark_start(m, st);
  TV_CUDA(cudaLaunchCooperativeKernel(kern, dim3(P.G), dim3(P.block), args, dyn, st));
  mark_end(m, st);
  m->last_launches += 1;
  return TV_OK;
}

// Picks and launches the kernel for one sequence on the device.
int launch_single(tv_model_s* m, const int32_t* obs_dev, int64_t T, int32_t* path_dev, double* ll_dev,
                  cudaStream_t st) {
  if (T < m->D)
    return fail(TV_ESHORT, "T=" + std::to_string(T) + " < D=" + std::to_string(m->D) +
                               "; the reference initialisation needs T >= D");
  int dev = 0;
  TV_CUDA(cudaGetDevice(&dev));
  int smem_optin = 0;
  TV_CUDA(cudaDeviceGetAttribute(&smem_optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev));
  const tv::CtaLayout L = tv::make_cta_layout(m->N, m->D);
  const bool cta_fits = L.bytes + 64 <= (size_t)smem_optin;
  int want = m->path_pref;
  if (want == TV_PATH_GRID_L2) want = TV_PATH_GRID;
  if (want == TV_PATH_AUTO) want = cta_fits ? TV_PATH_CTA : TV_PATH_GRID;
  if (want == TV_PATH_GRID) {
    int per_sm = 0;
    int G = m->sm_count;
    if (m->grid_ctas > 0) G = std::min(G, m->grid_ctas);
    const int force_l2 = m->path_pref == TV_PATH_GRID_L2 ? 1 : 0;
    if (m->plan_key_N != m->N || m->plan_key_D != m->D || m->plan_key_G != G || m->plan_key_L2 != force_l2) {
      std::vector<int> first, count, base;
      std::vector<long long> wr;
      tv::GridParams P;
      if (!plan_grid(m, G, smem_optin, force_l2 != 0, P, wr, first, count, base)) {
        if (m->path_pref == TV_PATH_GRID || m->path_pref == TV_PATH_GRID_L2)
          return fail(TV_EINVAL, "the grid kernel cannot take this shape (needs D > 8, D <= 65535, N small enough for the head CTA's tables and roles, about N <= 100)");
        want = TV_PATH_CTA;
      } else {
        const size_t dyn = std::max(P.w_bytes, P.h_bytes);
        const void* kern = grid_kernel_for(P);
        int rc;
        if ((rc = raise_smem_limit(kern)) != TV_OK) return rc;
        TV_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, P.block, dyn));
        if (per_sm < 1) return fail(TV_EINVAL, "grid kernel does not fit on an SM");
        if ((rc = m->seg_first.ensure(first.size())) != TV_OK) return rc;
        if ((rc = m->seg_count.ensure(count.size())) != TV_OK) return rc;
        if ((rc = m->seg_base.ensure(base.size())) != TV_OK) return rc;
        if ((rc = m->wrange.ensure(wr.size())) != TV_OK) return rc;
        TV_CUDA(upload(m->wrange.p, wr.data(), sizeof(long long) * wr.size()));
        TV_CUDA(upload(m->seg_first.p, first.data(), sizeof(int) * first.size()));
        TV_CUDA(upload(m->seg_count.p, count.data(), sizeof(int) * count.size()));
        TV_CUDA(upload(m->seg_base.p, base.data(), sizeof(int) * base.size()));
        m->plan = P;
        m->plan_key_N = m->N;
        m->plan_key_D = m->D;
        m->plan_key_G = G;
        m->plan_key_L2 = force_l2;
      }
    }
    if (want == TV_PATH_GRID) {
      m->last_path = TV_PATH_GRID;
      return launch_grid(m, obs_dev, T, path_dev, ll_dev, st, m->plan);
    }
  }
  m->last_path = TV_PATH_CTA;
  const int64_t off[2] = {0, T};
  return launch_batch(m, 1, off, obs_dev, path_dev, ll_dev, st);
}

int read_grid_status(tv_model_s* m, cudaStream_t st) {
  int s[4] = {0, 0, 0, 0};
  TV_CUDA(cudaMemcpyAsync(s, m->gflags.p, sizeof(int) * 4, cudaMemcpyDeviceToHost, st));
  TV_CUDA(cudaStreamSynchronize(st));
  if (s[2] == tv::TV_ETIMEOUT_DEV) {
    static const char* sites[] = {"?", "head waiting for worker partials", "worker waiting for a slot message",
                                  "worker re-scoring waiting for an exact score", "worker tail waiting for an exact score",
                                  "head waiting for tail partials", "head waiting for a window-sum copy"};
    const int k = (s[0] >= 1 && s[0] <= 6) ? s[0] : 0;
    return fail(TV_ETIMEOUT, std::string("grid decode: a bounded wait between CTAs timed out (") + sites[k] + ")");
  }
  if (s[2] == TV_ERANGE) return fail(TV_ERANGE, "an observation is outside [0, O)");
  if (s[2] != 0) return fail(TV_EINTERNAL, "grid decode: device back-pointer check failed");
  return TV_OK;
}

int read_status(tv_model_s* m, int n_seq, cudaStream_t st) {
  std::vector<int> s((size_t)n_seq);
  TV_CUDA(cudaMemcpyAsync(s.data(), m->status.p, sizeof(int) * n_seq, cudaMemcpyDeviceToHost, st));
  TV_CUDA(cudaStreamSynchronize(st));
  for (int k = 0; k < n_seq; ++k) {
    if (s[k] == TV_ERANGE) return fail(TV_ERANGE, "sequence " + std::to_string(k) + " has an observation outside [0, O)");
    if (s[k] != 0) return fail(TV_EINTERNAL, "device back-pointer check failed for sequence " + std::to_string(k));
  }
  return TV_OK;
}

// Device buffers freed together when the arena goes out of scope.
struct DevArena {
  std::vector<void*> p;
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  DevArena() = default;
  DevArena(const DevArena&) = delete;
  DevArena& operator=(const DevArena&) = delete;
  ~DevArena() {
    for (void* q : p) cudaFree(q);
    if (e0) cudaEventDestroy(e0);
    if (e1) cudaEventDestroy(e1);
  }
  template <class T>
  int get(T** out, size_t n) {
    void* q = nullptr;
    if (cudaMalloc(&q, sizeof(T) * std::max<size_t>(n, 1)) != cudaSuccess) {
      cudaGetLastError();
      return TV_ENOMEM;
    }
    p.push_back(q);
    *out = (T*)q;
    return TV_OK;
  }
};

// Device time of the calling thread's last forward-backward kernel (CUDA
// events around the launch).
thread_local double g_fb_kernel_ms = 0.0;

// The forward-backward E step (tv_fb): device copies of the inputs and
// outputs, one launch, copies back.
int fb_run(int censoring, int64_t tau, int J, int M, const double* d, const double* p, const double* pi,
           const double* pdf, double* F, double* L, double* G, double* L1, double* Nn, double* Norm,
           double* eta) {
  if (censoring != 0 && censoring != 1)
    return fail(TV_EINVAL, "tv_fb: censoring must be 0 (none) or 1 (right); left censoring (2) is not supported");
  if (tau < 1 || tau > 0x7fffffffLL || J < 1 || J > 1024 || M < 1)
    return fail(TV_EINVAL, "tv_fb: need tau >= 1, 1 <= J <= 1024, M >= 1");
  if (!d || !p || !pi || !pdf || !F || !L || !G || !L1 || !Nn || !Norm || !eta)
    return fail(TV_EINVAL, "tv_fb: null argument");
  int devs = 0;
  if (cudaGetDeviceCount(&devs) != cudaSuccess || devs == 0) return fail(TV_ENODEV, "no CUDA device");
  const size_t JT = (size_t)J * (size_t)tau, JM = (size_t)J * M;
  DevArena b;
  double *dd, *dp, *dpi, *dpdf, *dF, *dL, *dG, *dL1, *dN, *dNorm, *deta, *dS, *dD, *dring = nullptr;
  int* dst;
  if (b.get(&dd, JM) || b.get(&dp, (size_t)J * J) || b.get(&dpi, J) || b.get(&dpdf, JT) || b.get(&dF, JT) ||
      b.get(&dL, JT) || b.get(&dG, JT) || b.get(&dL1, JT) || b.get(&dN, (size_t)tau) || b.get(&dNorm, JT) ||
      b.get(&deta, JM) || b.get(&dS, JT) || b.get(&dD, (size_t)J * (M + 1)) || b.get(&dst, 1))
    return fail(TV_ENOMEM, "tv_fb: device allocation failed");
  int dev = 0, smem_optin = 0;
  TV_CUDA(cudaGetDevice(&dev));
  TV_CUDA(cudaDeviceGetAttribute(&smem_optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev));
  // J <= 32: the short-chain kernel (a warp per state, the ratios and eta
  // weights kept for the backward pass), with the window in registers up to
  // 32 * FB_REG_BLOCKS durations and in rings (forward, backward, eta
  // accumulators) beyond; otherwise the general one
  const bool small = J <= 32;
  const bool regs = small && M <= 32 * tv::FB_REG_BLOCKS;
  const size_t nrings = regs ? 0 : small ? 3 : 2;
  const size_t ring_bytes = nrings * JM * sizeof(double);
  const bool in_smem = ring_bytes + 2048 <= (size_t)smem_optin;
  if (!in_smem && b.get(&dring, nrings * JM)) return fail(TV_ENOMEM, "tv_fb: device allocation failed");
  double *dR = nullptr, *dA = nullptr, *dQ = nullptr, *dpart = nullptr;
  if (small && (b.get(&dR, JT) || b.get(&dA, JT))) return fail(TV_ENOMEM, "tv_fb: device allocation failed");
  // register path: eta's window terms in chunks of t over the whole GPU
  // (about eight warps per SM, chunks of at least 4 M steps)
  long long chunk = 1;
  int nchunks = 1;
  if (regs) {
    int sms = 1;
    TV_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    const long long steps = std::max<long long>(1, (long long)tau - 1);
    chunk = std::max<long long>(4LL * M, (steps * J + 8LL * sms - 1) / (8LL * sms));
    nchunks = (int)((steps + chunk - 1) / chunk);
    if (b.get(&dQ, JT) || b.get(&dpart, (size_t)J * nchunks * M))
      return fail(TV_ENOMEM, "tv_fb: device allocation failed");
  }
  TV_CUDA(cudaMemcpy(dd, d, sizeof(double) * JM, cudaMemcpyHostToDevice));
  TV_CUDA(cudaMemcpy(dp, p, sizeof(double) * J * J, cudaMemcpyHostToDevice));
  TV_CUDA(cudaMemcpy(dpi, pi, sizeof(double) * J, cudaMemcpyHostToDevice));
  TV_CUDA(cudaMemcpy(dpdf, pdf, sizeof(double) * JT, cudaMemcpyHostToDevice));
  // the columns the recursions do not write stay as the caller passed them
  // (hsmmlearn hands in zeroed arrays): G[:, 0], L1[:, tau-1]
  TV_CUDA(cudaMemcpy(dG, G, sizeof(double) * JT, cudaMemcpyHostToDevice));
  TV_CUDA(cudaMemcpy(dL1, L1, sizeof(double) * JT, cudaMemcpyHostToDevice));
  TV_CUDA(cudaMemset(dS, 0, sizeof(double) * JT));
  tv::FbArgs A{};
  A.censoring = censoring; A.tau = (int)tau; A.J = J; A.M = M;
  A.d = dd; A.p = dp; A.pi = dpi; A.pdf = dpdf;
  A.F = dF; A.L = dL; A.G = dG; A.L1 = dL1; A.N = dN; A.Norm = dNorm; A.eta = deta;
  A.S = dS; A.D = dD; A.ring = dring; A.rings_in_smem = in_smem ? 1 : 0; A.status = dst;
  A.R = dR; A.A = dA; A.Q = dQ; A.part = dpart; A.chunk = chunk; A.nchunks = nchunks;
  const int threads = 32 * std::min(32, J);
  const size_t dyn = in_smem ? ring_bytes : 0;
  constexpr int KR = tv::FB_REG_BLOCKS;
  const void* kern = !small ? (const void*)tv::fb_kernel
                     : !regs ? (const void*)tv::fb_small_kernel<0, 1024>
                     : J <= 16 ? (const void*)tv::fb_small_kernel<KR, 512> : (const void*)tv::fb_small_kernel<KR, 1024>;
  if (dyn) {
    int rc = raise_smem_limit(kern);
    if (rc != TV_OK) return rc;
  }
  TV_CUDA(cudaEventCreate(&b.e0));
  TV_CUDA(cudaEventCreate(&b.e1));
  TV_CUDA(cudaEventRecord(b.e0));
  if (!small) tv::fb_kernel<<<1, threads, dyn>>>(A);
  else if (!regs) tv::fb_small_kernel<0, 1024><<<1, threads, dyn>>>(A);
  else if (J <= 16) tv::fb_small_kernel<KR, 512><<<1, threads, dyn>>>(A);
  else tv::fb_small_kernel<KR, 1024><<<1, threads, dyn>>>(A);
  if (regs) {
    TV_CUDA(cudaGetLastError());
    tv::fb_eta_chunk_kernel<KR><<<dim3(nchunks, J), 32>>>(A);
    TV_CUDA(cudaGetLastError());
    tv::fb_eta_final_kernel<<<J, 128>>>(A);
  }
  TV_CUDA(cudaGetLastError());
  TV_CUDA(cudaEventRecord(b.e1));
  TV_CUDA(cudaEventSynchronize(b.e1));
  float kms = 0.0f;
  TV_CUDA(cudaEventElapsedTime(&kms, b.e0, b.e1));
  g_fb_kernel_ms = (double)kms;
  int st = 0;
  TV_CUDA(cudaMemcpy(&st, dst, sizeof(int), cudaMemcpyDeviceToHost));
  TV_CUDA(cudaMemcpy(F, dF, sizeof(double) * JT, cudaMemcpyDeviceToHost));
  TV_CUDA(cudaMemcpy(L, dL, sizeof(double) * JT, cudaMemcpyDeviceToHost));
  TV_CUDA(cudaMemcpy(G, dG, sizeof(double) * JT, cudaMemcpyDeviceToHost));
  TV_CUDA(cudaMemcpy(L1, dL1, sizeof(double) * JT, cudaMemcpyDeviceToHost));
  TV_CUDA(cudaMemcpy(Nn, dN, sizeof(double) * tau, cudaMemcpyDeviceToHost));
  TV_CUDA(cudaMemcpy(Norm, dNorm, sizeof(double) * JT, cudaMemcpyDeviceToHost));
  TV_CUDA(cudaMemcpy(eta, deta, sizeof(double) * JM, cudaMemcpyDeviceToHost));
  if (st != 0)
    return fail(TV_ENONPOS, "forward-backward: a normaliser or forward variable is not positive");
  return TV_OK;
}


}  // namespace

// ---------------------------------------------------------------------------
// Fixed-scratch decode (tv_decode_device_static): the one-CTA kernel with all
// of its global scratch carved out of this file-scope array, so the call
// allocates nothing.  Host code must not use the array's name as an address
// (it is a host-side stand-in); the device address is looked up once per
// device with cudaGetSymbolAddress.
// ---------------------------------------------------------------------------
static __device__ __align__(256) unsigned char g_static_scratch[TV_STATIC_SCRATCH_BYTES];

namespace {

std::mutex g_static_mu;
constexpr int kMaxDevices = 64;
unsigned char* g_static_ptr[kMaxDevices] = {};

// Start-of-call reset of the control words this call relies on: the work
// queue counter and the status must start at zero (the array keeps whatever
// the previous call left).
__global__ void static_reset_kernel(int64_t* off, long long T, int* counter, int* status) {
  off[0] = 0;
  off[1] = T;
  *counter = 0;
  *status = 0;
}

__global__ void static_status_kernel(const int* status, int* out) { *out = *status; }

int static_scratch_for_current_device(unsigned char** out) {
  int dev = 0;
  TV_CUDA(cudaGetDevice(&dev));
  if (dev < 0 || dev >= kMaxDevices) return fail(TV_EINVAL, "device ordinal out of range");
  std::lock_guard<std::mutex> lk(g_static_mu);
  if (!g_static_ptr[dev]) {
    void* p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_static_scratch);
    if (e != cudaSuccess || !p)
      return fail(TV_ECUDA, std::string("cudaGetSymbolAddress(static scratch): ") + cudaGetErrorString(e));
    const int rc = raise_smem_limit((const void*)tv::cta_decode_kernel<kThreads>);
    if (rc != TV_OK) return rc;
    g_static_ptr[dev] = (unsigned char*)p;
  }
  *out = g_static_ptr[dev];
  return TV_OK;
}


// Finite check and max |x| of a device table (the emission table built on the
// device by the Gaussian front-end): out[0] = bits of max |x| (non-negative
// doubles order as their bit patterns), out[1] = 1 if any entry is not finite.
__global__ void absmax_kernel(const double* __restrict__ a, size_t n, unsigned long long* out) {
  unsigned long long mx = 0;
  unsigned long long bad = 0;
  for (size_t k = blockIdx.x * (size_t)blockDim.x + threadIdx.x; k < n; k += (size_t)gridDim.x * blockDim.x) {
    const double v = a[k];
    if (!isfinite(v)) bad = 1;
    else mx = max(mx, (unsigned long long)__double_as_longlong(fabs(v)));
  }
  for (int o = 16; o > 0; o >>= 1) {
    mx = max(mx, __shfl_xor_sync(0xffffffffu, mx, o));
    bad |= __shfl_xor_sync(0xffffffffu, bad, o);
  }
  if ((threadIdx.x & 31) == 0) {
    atomicMax(out, mx);
    if (bad) atomicOr(out + 1, 1ull);
  }
}

// Gaussian emission front-end: table[t][j] = log N(x_t; mu_j, sd_j)
// = ((-0.5 * z) * z - log sd_j) - log(2 pi)/2 with z = (x_t - mu_j) / sd_j,
// each operation rounded once (no fused multiply-add), so the table equals
// the same expression evaluated in FP64 on the host given the same log sd_j
// and constant (computed on the host with the C library's log).
__global__ void gaussian_loglik_kernel(const double* __restrict__ x, long long T, int N, const double* __restrict__ mu,
                                       const double* __restrict__ sd, const double* __restrict__ logsd, double c,
                                       double* __restrict__ table) {
  const long long n = T * N;
  for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < n; k += (long long)gridDim.x * blockDim.x) {
    const long long t = k / N;
    const int j = (int)(k - t * N);
    const double z = __ddiv_rn(__dsub_rn(x[t], mu[j]), sd[j]);
    table[k] = __dsub_rn(__dsub_rn(__dmul_rn(__dmul_rn(-0.5, z), z), logsd[j]), c);
  }
}

__global__ void iota_kernel(int32_t* a, long long n) {
  for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < n; k += (long long)gridDim.x * blockDim.x)
    a[k] = (int32_t)k;
}

// The model from host tables (emission given on the host, or already on the
// device in em_dev with its max |x| in emax_dev); uploads on the thread's
// allocation stream when set.
int model_create_impl(int N, int O, int D, const double* trans, const double* emission, const double* em_dev,
                      const double* start, const double* dur, tv_model* out, double emax_dev = 0.0) {
  if (!out) return fail(TV_EINVAL, "out is null");
  *out = nullptr;
  if (N <= 0 || O <= 0 || D <= 0) return fail(TV_EINVAL, "n_states, n_symbols and max_dur must be positive");
  if (N > 32768 || D > 65536) return fail(TV_ETOOBIG, "n_states must be <= 32768 and max_dur <= 65536");
  if (!trans || !start || !dur || (!emission && !em_dev)) return fail(TV_EINVAL, "null model table");
  tv_model_s* m = new tv_model_s();
  m->N = N; m->O = O; m->D = D;
  bool ok = all_finite(trans, (size_t)N * N, &m->tmax) && all_finite(start, (size_t)N, &m->smax) &&
            all_finite(dur, (size_t)D * N, &m->dmax);
  if (emission) ok = ok && all_finite(emission, (size_t)O * N, &m->emax);
  else m->emax = emax_dev;
  if (!ok) {
    delete m;
    return fail(TV_ENONFINITE, "model tables must be finite (log(p + 1e-30) as in HSMM.to_log_space)");
  }
  int devs = 0;
  if (cudaGetDeviceCount(&devs) != cudaSuccess || devs == 0) {
    delete m;
    return fail(TV_ENODEV, "no CUDA device");
  }
  int dev = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&m->sm_count, cudaDevAttrMultiProcessorCount, dev);
  std::vector<double> durT((size_t)N * D), survT;
  for (int j = 0; j < N; ++j)
    for (int d = 0; d < D; ++d) durT[(size_t)j * D + d] = dur[(size_t)d * N + j];
  survival_T(N, D, dur, survT);
  int rc = TV_OK;
  if ((rc = m->em.ensure((size_t)O * N)) || (rc = m->trans.ensure((size_t)N * N)) ||
      (rc = m->start.ensure((size_t)N)) || (rc = m->durT.ensure((size_t)N * D)) ||
      (rc = m->survT.ensure((size_t)N * D))) {
    tv_model_destroy(m);
    return rc;
  }
  cudaError_t e = cudaSuccess;
  if (emission) {
    e = upload(m->em.p, emission, sizeof(double) * O * N);
  } else {
    e = g_alloc_async ? cudaMemcpyAsync(m->em.p, em_dev, sizeof(double) * O * N, cudaMemcpyDeviceToDevice, g_alloc_stream)
                      : cudaMemcpy(m->em.p, em_dev, sizeof(double) * O * N, cudaMemcpyDeviceToDevice);
  }
  if (e == cudaSuccess) e = upload(m->trans.p, trans, sizeof(double) * N * N);
  if (e == cudaSuccess) e = upload(m->start.p, start, sizeof(double) * N);
  if (e == cudaSuccess) e = upload(m->durT.p, durT.data(), sizeof(double) * N * D);
  if (e == cudaSuccess) e = upload(m->survT.p, survT.data(), sizeof(double) * N * D);
  if (e != cudaSuccess) {
    tv_model_destroy(m);
    return fail(TV_ECUDA, std::string("model upload: ") + cudaGetErrorString(e));
  }
  *out = m;
  return TV_OK;
}

// The Gaussian front-end into a device table (T x N), on `st`.
int gaussian_table(const double* x_dev, int64_t T, int N, const double* mean, const double* sd, double* table_dev,
                   cudaStream_t st) {
  if (!x_dev || !mean || !sd || !table_dev || T <= 0 || N <= 0) return fail(TV_EINVAL, "bad argument");
  std::vector<double> par((size_t)3 * N);
  for (int j = 0; j < N; ++j) {
    if (!(sd[j] > 0.0) || !std::isfinite(sd[j]) || !std::isfinite(mean[j]))
      return fail(TV_EINVAL, "Gaussian means must be finite and standard deviations positive");
    par[j] = mean[j];
    par[(size_t)N + j] = sd[j];
    par[(size_t)2 * N + j] = std::log(sd[j]);
  }
  const double c = 0.5 * std::log(2.0 * 3.141592653589793);
  double* par_dev = nullptr;
  TV_CUDA(cudaMallocAsync((void**)&par_dev, sizeof(double) * 3 * N, st));
  TV_CUDA(cudaMemcpyAsync(par_dev, par.data(), sizeof(double) * 3 * N, cudaMemcpyHostToDevice, st));
  const long long n = (long long)T * N;
  const int blocks = (int)std::min<long long>((n + 255) / 256, 4096);
  gaussian_loglik_kernel<<<blocks, 256, 0, st>>>(x_dev, T, N, par_dev, par_dev + N, par_dev + 2 * N, c, table_dev);
  TV_CUDA(cudaGetLastError());
  TV_CUDA(cudaFreeAsync(par_dev, st));
  return TV_OK;
}

// A model whose emission table is built on the device from float64
// observations x (host, T) and per-state Gaussian mean / sd: emission row t
// is observation t, so the decode takes obs = 0..T-1.
int model_create_gaussian(int N, int D, int64_t T, const double* trans, const double* start, const double* dur,
                          const double* x, const double* mean, const double* sd, tv_model* out) {
  if (!out) return fail(TV_EINVAL, "out is null");
  *out = nullptr;
  if (T <= 0 || T > 0x7fffffffLL || N <= 0) return fail(TV_EINVAL, "bad sizes");
  if (!x || !mean || !sd) return fail(TV_EINVAL, "null Gaussian argument");
  for (int64_t t = 0; t < T; ++t)
    if (!std::isfinite(x[t])) return fail(TV_ENONFINITE, "observations must be finite");
  cudaStream_t st = g_alloc_async ? g_alloc_stream : (cudaStream_t)0;
  double* x_dev = nullptr;
  double* table = nullptr;
  unsigned long long* red = nullptr;
  auto cleanup = [&]() {
    if (x_dev) cudaFreeAsync(x_dev, st);
    if (table) cudaFreeAsync(table, st);
    if (red) cudaFreeAsync(red, st);
  };
  cudaError_t e = cudaMallocAsync((void**)&x_dev, sizeof(double) * T, st);
  if (e == cudaSuccess) e = cudaMallocAsync((void**)&table, sizeof(double) * T * N, st);
  if (e == cudaSuccess) e = cudaMallocAsync((void**)&red, sizeof(unsigned long long) * 2, st);
  if (e != cudaSuccess) {
    cudaGetLastError();
    cleanup();
    return fail(TV_ENOMEM, std::string("device allocation: ") + cudaGetErrorString(e));
  }
  e = cudaMemcpyAsync(x_dev, x, sizeof(double) * T, cudaMemcpyHostToDevice, st);
  int rc = e == cudaSuccess ? gaussian_table(x_dev, T, N, mean, sd, table, st)
                            : fail(TV_ECUDA, std::string("upload: ") + cudaGetErrorString(e));
  unsigned long long hr[2] = {0, 0};
  if (rc == TV_OK) {
    e = cudaMemsetAsync(red, 0, sizeof(unsigned long long) * 2, st);
    if (e == cudaSuccess) {
      absmax_kernel<<<256, 256, 0, st>>>(table, (size_t)T * N, red);
      e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaMemcpyAsync(hr, red, sizeof(hr), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) rc = fail(TV_ECUDA, std::string("Gaussian front-end: ") + cudaGetErrorString(e));
  }
  if (rc == TV_OK) {
    double emax = 0.0;
    std::memcpy(&emax, &hr[0], sizeof(double));
    if (hr[1]) rc = fail(TV_ENONFINITE, "the Gaussian log-likelihood table is not finite");
    else rc = model_create_impl(N, (int)T, D, trans, nullptr, table, start, dur, out, emax);
  }
  cleanup();
  return rc;
}

}  // namespace

extern "C" {

const char* tv_last_error(void) { return g_err.c_str(); }

int tv_model_create(int N, int O, int D, const double* trans, const double* emission,
                    const double* dur_lin, const double* start, const double* dur, tv_model* out) {
  (void)dur_lin;
  if (!emission) return fail(TV_EINVAL, "null model table");
  return model_create_impl(N, O, D, trans, emission, nullptr, start, dur, out);
}

int tv_model_destroy(tv_model m) {
  if (!m) return TV_OK;
  m->em.release(); m->trans.release(); m->start.release(); m->durT.release(); m->survT.release();
  m->qem.release(); m->qtr.release(); m->qdurT.release();
  m->psi.release(); m->status.release(); m->counter.release(); m->off.release(); m->order.release(); m->scratch.release();
  m->msgs.release(); m->dinit.release(); m->ck.release(); m->hwin.release(); m->wrange.release(); m->wglob.release();
  m->seg_first.release(); m->seg_count.release(); m->seg_base.release(); m->gflags.release();
  if (m->ev0) cudaEventDestroy(m->ev0);
  if (m->ev1) cudaEventDestroy(m->ev1);
  m->obs_tmp.release(); m->path_tmp.release(); m->ll_tmp.release();
  delete m;
  return TV_OK;
}

int64_t tv_model_last_launches(tv_model m) { return m ? m->last_launches : 0; }

int tv_model_set_path(tv_model m, int path, int grid_ctas) {
  if (!m || path < TV_PATH_AUTO || path > TV_PATH_GRID_L2 || grid_ctas < 0) return fail(TV_EINVAL, "bad path option");
  std::lock_guard<std::mutex> lk(m->mu);
  m->path_pref = path;
  m->grid_ctas = grid_ctas;
  return TV_OK;
}

int tv_model_last_path(tv_model m) { return m ? m->last_path : 0; }

int tv_model_batch_threads(tv_model m) { return m ? m->batch_threads : 0; }

int tv_model_batch_grid(tv_model m) { return m ? m->batch_grid : 0; }

int tv_model_drop_partial(tv_model m, int64_t step, int segment) {
  if (!m || step < 1 || step > 0xffffffffLL || segment < 0) return fail(TV_EINVAL, "bad argument");
  m->drop_tag = (unsigned)step;
  m->drop_seg = segment;
  return TV_OK;
}

int tv_grid_plan_info(int N, int D, int G, int smem_optin, int force_l2, int64_t* out) {
  if (!out) return fail(TV_EINVAL, "null argument");
  for (int k = 0; k < 10; ++k) out[k] = 0;
  if (N <= 0 || D <= 0 || G <= 0 || smem_optin <= 0) return fail(TV_EINVAL, "N, D, G and the shared-memory limit must be positive");
  tv::GridParams P{};
  std::vector<long long> wr;
  std::vector<int> first, count, base;
  if (!plan_grid_nd(N, D, G, smem_optin, force_l2 != 0, P, wr, first, count, base)) return TV_OK;
  out[0] = 1;
  out[1] = P.block;
  out[2] = (int64_t)std::max(P.w_bytes, P.h_bytes);
  out[3] = P.w_global;
  out[4] = P.cs_split;
  out[5] = P.S;
  out[6] = P.max_seg;
  out[7] = (int64_t)P.cs_threads * (1 + P.cs_split) + 2 * P.st_threads + P.in_threads;
  out[8] = P.w_qd_smem;
  int busy = 0;
  for (int w = 0; w + 1 < G; ++w) busy += wr[2 * w] < wr[2 * w + 1] ? 1 : 0;
  out[9] = busy;
  return TV_OK;
}

int tv_model_set_timing(tv_model m, int enable) {
  if (!m) return fail(TV_EINVAL, "null model");
  std::lock_guard<std::mutex> lk(m->mu);
  if (enable && !m->ev0) {
    TV_CUDA(cudaEventCreate(&m->ev0));
    TV_CUDA(cudaEventCreate(&m->ev1));
  }
  m->timing = enable != 0;
  m->timed = false;
  return TV_OK;
}

double tv_model_kernel_ms(tv_model m) {
  if (!m || !m->timed) return -1.0;
  if (cudaEventSynchronize(m->ev1) != cudaSuccess) return -1.0;
  float ms = 0.f;
  if (cudaEventElapsedTime(&ms, m->ev0, m->ev1) != cudaSuccess) return -1.0;
  return (double)ms;
}

int tv_decode_device(tv_model m, const int32_t* obs_dev, int64_t T, int32_t* path_dev, double* ll_dev,
                     void* stream) {
  if (!m || !obs_dev || !path_dev) return fail(TV_EINVAL, "null argument");
  if (T <= 0 || T > 0x7fffffffLL) return fail(TV_ETOOBIG, "T must be in [1, 2^31-1]");
  std::lock_guard<std::mutex> lk(m->mu);
  m->last_launches = 0;
  return launch_single(m, obs_dev, T, path_dev, ll_dev, (cudaStream_t)stream);
}

int tv_decode(tv_model m, const int32_t* obs, int64_t T, int32_t* path_out, double* loglik_out) {
  if (!m || !obs || !path_out) return fail(TV_EINVAL, "null argument");
  if (T <= 0 || T > 0x7fffffffLL) return fail(TV_ETOOBIG, "T must be in [1, 2^31-1]");
  int rc = check_obs_host(obs, T, m->O);
  if (rc != TV_OK) return rc;
  std::lock_guard<std::mutex> lk(m->mu);
  m->last_launches = 0;
  cudaStream_t st = 0;
  if ((rc = m->obs_tmp.ensure((size_t)T)) != TV_OK) return rc;
  if ((rc = m->path_tmp.ensure((size_t)T)) != TV_OK) return rc;
  if ((rc = m->ll_tmp.ensure(1)) != TV_OK) return rc;
  TV_CUDA(cudaMemcpyAsync(m->obs_tmp.p, obs, sizeof(int32_t) * T, cudaMemcpyHostToDevice, st));
  if ((rc = launch_single(m, m->obs_tmp.p, T, m->path_tmp.p, m->ll_tmp.p, st)) != TV_OK) return rc;
  TV_CUDA(cudaMemcpyAsync(path_out, m->path_tmp.p, sizeof(int32_t) * T, cudaMemcpyDeviceToHost, st));
  double ll = 0;
  TV_CUDA(cudaMemcpyAsync(&ll, m->ll_tmp.p, sizeof(double), cudaMemcpyDeviceToHost, st));
  rc = (m->last_path == TV_PATH_GRID) ? read_grid_status(m, st) : read_status(m, 1, st);
  if (rc != TV_OK) return rc;
  if (loglik_out) *loglik_out = ll;
  return TV_OK;
}

int tv_decode_batch_device(tv_model m, int n_seq, const int64_t* offsets, const int32_t* obs_dev,
                           int32_t* path_dev, double* ll_dev, void* stream) {
  if (!m || !offsets || !obs_dev || !path_dev || n_seq <= 0) return fail(TV_EINVAL, "bad argument");
  std::lock_guard<std::mutex> lk(m->mu);
  m->last_launches = 0;
  if (offsets[0] != 0) return fail(TV_EINVAL, "offsets[0] must be 0");
  return launch_batch(m, n_seq, offsets, obs_dev, path_dev, ll_dev, (cudaStream_t)stream, true);
}

int tv_decode_batch(tv_model m, int n_seq, const int64_t* offsets, const int32_t* obs, int32_t* path,
                    double* loglik_out) {
  if (!m || !offsets || !obs || !path || n_seq <= 0) return fail(TV_EINVAL, "bad argument");
  if (offsets[0] != 0) return fail(TV_EINVAL, "offsets[0] must be 0");
  for (int k = 0; k < n_seq; ++k)
    if (offsets[k + 1] <= offsets[k]) return fail(TV_EINVAL, "offsets must increase");
  const int64_t total = offsets[n_seq];
  // Observations are range-checked by the kernel, per sequence, before any
  // table lookup (a bad sequence is reported as TV_ERANGE with its index),
  // so a batch gets no serial host pass over all of its observations.
  int rc;
  std::lock_guard<std::mutex> lk(m->mu);
  m->last_launches = 0;
  cudaStream_t st = 0;
  if ((rc = m->obs_tmp.ensure((size_t)total)) != TV_OK) return rc;
  if ((rc = m->path_tmp.ensure((size_t)total)) != TV_OK) return rc;
  if ((rc = m->ll_tmp.ensure((size_t)n_seq)) != TV_OK) return rc;
  TV_CUDA(cudaMemcpyAsync(m->obs_tmp.p, obs, sizeof(int32_t) * total, cudaMemcpyHostToDevice, st));
  if ((rc = launch_batch(m, n_seq, offsets, m->obs_tmp.p, m->path_tmp.p, m->ll_tmp.p, st, true)) != TV_OK)
    return rc;
  TV_CUDA(cudaMemcpyAsync(path, m->path_tmp.p, sizeof(int32_t) * total, cudaMemcpyDeviceToHost, st));
  std::vector<double> ll((size_t)n_seq);
  TV_CUDA(cudaMemcpyAsync(ll.data(), m->ll_tmp.p, sizeof(double) * n_seq, cudaMemcpyDeviceToHost, st));
  if ((rc = read_status(m, n_seq, st)) != TV_OK) return rc;
  if (loglik_out) std::memcpy(loglik_out, ll.data(), sizeof(double) * n_seq);
  return TV_OK;
}

int tv_decode_tensor_viterbi_cuda(int n_states, int n_symbols, int max_dur, int64_t T, const double* trans,
                                  const double* emission, const double* dur_lin, const double* start,
                                  const double* dur, const int32_t* obs, int32_t* path_out,
                                  double* loglik_out) {
  tv_model m = nullptr;
  int rc = tv_model_create(n_states, n_symbols, max_dur, trans, emission, dur_lin, start, dur, &m);
  if (rc != TV_OK) return rc;
  rc = tv_decode(m, obs, T, path_out, loglik_out);
  std::string keep = g_err;
  tv_model_destroy(m);
  g_err = keep;
  return rc;
}


int tv_decode_device_static(tv_model m, const int32_t* obs_dev, int64_t T, int32_t* path_dev, double* ll_dev,
                            int* status_dev, void* stream) {
  if (!m || !obs_dev || !path_dev) return fail(TV_EINVAL, "null argument");
  if (T <= 0 || T > 0x7fffffffLL) return fail(TV_ETOOBIG, "T must be in [1, 2^31-1]");
  const int N = m->N, O = m->O, D = m->D;
  if (T < D)
    return fail(TV_ESHORT, "T=" + std::to_string(T) + " < D=" + std::to_string(D) +
                               "; the reference initialisation needs T >= D");
  // Carve the scratch: quantised tables, offsets + control words, back-pointers.
  auto al = [](unsigned long long x) { return (x + 255ull) & ~255ull; };
  const unsigned long long o_qem = 0;
  const unsigned long long o_qtr = al(o_qem + 8ull * O * N);
  const unsigned long long o_qd = al(o_qtr + 8ull * N * N);
  const unsigned long long o_ctl = al(o_qd + 8ull * N * D);
  const unsigned long long o_psi = al(o_ctl + 64);
  const unsigned long long need = o_psi + 4ull * (unsigned long long)T * N;
  if (need > TV_STATIC_SCRATCH_BYTES)
    return fail(TV_ETOOBIG, "problem needs " + std::to_string(need) + " bytes of scratch; the fixed-scratch entry "
                            "point has " + std::to_string((unsigned long long)TV_STATIC_SCRATCH_BYTES) +
                            " (use tv_decode_device)");
  int dev = 0;
  TV_CUDA(cudaGetDevice(&dev));
  int smem_optin = 0;
  TV_CUDA(cudaDeviceGetAttribute(&smem_optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev));
  tv::CtaLayout L = tv::make_cta_layout(N, D);
  if (L.bytes + 64 > (unsigned long long)smem_optin)
    return fail(TV_ETOOBIG, "the D-deep window does not fit one CTA's shared memory; the fixed-scratch entry "
                            "point decodes windows up to 34*N*D + 8*N*N = " + std::to_string(smem_optin - 64) +
                            " bytes (use tv_decode_device)");
  L.in_smem = 1;
  unsigned char* base = nullptr;
  int rc = static_scratch_for_current_device(&base);
  if (rc != TV_OK) return rc;
  cudaStream_t st = (cudaStream_t)stream;
  long long* qem = (long long*)(base + o_qem);
  long long* qtr = (long long*)(base + o_qtr);
  long long* qd = (long long*)(base + o_qd);
  int64_t* off = (int64_t*)(base + o_ctl);
  int* counter = (int*)(base + o_ctl + 16);
  int* status = (int*)(base + o_ctl + 20);
  uint32_t* psi = (uint32_t*)(base + o_psi);
  const Quant Q = choose_quant(m, T);
  static_reset_kernel<<<1, 1, 0, st>>>(off, T, counter, status);
  quantize_kernel<<<64, 256, 0, st>>>(m->em.p, qem, (size_t)O * N, Q.scale);
  quantize_kernel<<<64, 256, 0, st>>>(m->trans.p, qtr, (size_t)N * N, Q.scale);
  quantize_kernel<<<64, 256, 0, st>>>(m->durT.p, qd, (size_t)N * D, Q.scale);
  tv::ModelView v = view(m, Q);
  v.qem = qem;
  v.qtr = qtr;
  v.qdurT = qd;
  tv::BatchView bv{};
  bv.obs = obs_dev;
  bv.off = off;
  bv.path = path_dev;
  bv.loglik = ll_dev;
  bv.psi = psi;
  bv.status = status;
  bv.next = counter;
  bv.order = nullptr;
  bv.n_seq = 1;
  tv::cta_decode_kernel<kThreads><<<1, kThreads, L.bytes, st>>>(v, bv, L, nullptr);
  if (status_dev) static_status_kernel<<<1, 1, 0, st>>>(status, status_dev);
  TV_CUDA(cudaGetLastError());
  return TV_OK;
}

int tv_fb(int censoring, int64_t tau, int J, int M, const double* d, const double* p, const double* pi,
          const double* pdf, double* F, double* L, double* G, double* L1, double* Nn, double* Norm,
          double* eta) {
  return fb_run(censoring, tau, J, M, d, p, pi, pdf, F, L, G, L1, Nn, Norm, eta);
}

double tv_fb_last_kernel_ms(void) { return g_fb_kernel_ms; }

int tv_fp64_peak(double* out) {
  if (!out) return fail(TV_EINVAL, "tv_fp64_peak: out is null");
  int devs = 0;
  if (cudaGetDeviceCount(&devs) != cudaSuccess || devs == 0) return fail(TV_ENODEV, "no CUDA device");
  DevArena b;
  double *din, *sink;
  unsigned long long* clk;
  if (b.get(&din, 16) || b.get(&sink, 1024) || b.get(&clk, 1)) return fail(TV_ENOMEM, "tv_fp64_peak: allocation");
  double h[16];
  for (int i = 0; i < 8; ++i) h[i] = 1.0 + 0.125 * i;
  h[8] = 0.999999;  // the chains converge to z / (1 - y): finite
  h[9] = 1e-3;
  for (int i = 10; i < 16; ++i) h[i] = 0.0;
  TV_CUDA(cudaMemcpy(din, h, sizeof h, cudaMemcpyHostToDevice));
  TV_CUDA(cudaEventCreate(&b.e0));
  TV_CUDA(cudaEventCreate(&b.e1));
  const int warps = 8;
  const long long iters = 1 << 15;
  unsigned long long hc = 0;
  // issue rate: 8 warps x 8 independent chains (warm-up launch first)
  for (int rep = 0; rep < 2; ++rep) {
    TV_CUDA(cudaMemset(clk, 0, sizeof(unsigned long long)));
    TV_CUDA(cudaEventRecord(b.e0));
    tv::fp64_issue_kernel<<<1, 32 * warps>>>(1, rep ? iters : 1024, din, sink, clk);
    TV_CUDA(cudaGetLastError());
    TV_CUDA(cudaEventRecord(b.e1));
    TV_CUDA(cudaEventSynchronize(b.e1));
  }
  TV_CUDA(cudaMemcpy(&hc, clk, sizeof hc, cudaMemcpyDeviceToHost));
  float ms = 0.0f;
  TV_CUDA(cudaEventElapsedTime(&ms, b.e0, b.e1));
  const double warp_insts = (double)warps * 8.0 * (double)iters;
  out[0] = warp_insts / (double)std::max(hc, 1ULL);                   // FP64 warp instructions per clock, one SM
  out[1] = warp_insts * 32.0 * 2.0 / ((double)ms * 1e-3);              // FLOP/s of one SM (an FMA is two)
  out[2] = (double)hc / ((double)ms * 1e-3) / 1e6;                     // SM clock over the run, MHz
  // dependent latency: one warp, one chain
  TV_CUDA(cudaMemset(clk, 0, sizeof(unsigned long long)));
  tv::fp64_issue_kernel<<<1, 32>>>(0, iters, din, sink, clk);
  TV_CUDA(cudaGetLastError());
  TV_CUDA(cudaDeviceSynchronize());
  TV_CUDA(cudaMemcpy(&hc, clk, sizeof hc, cudaMemcpyDeviceToHost));
  out[3] = (double)hc / (double)iters;                                 // clocks per dependent FP64 instruction
  return TV_OK;
}

int tv_step_floor(int n_states, int max_dur, int64_t steps, double* out) {
  if (!out || n_states < 1 || n_states > tv::GRID_MAX_N || max_dur < 1 || steps < 1)
    return fail(TV_EINVAL, "tv_step_floor: 1 <= n_states <= 128, max_dur >= 1, steps >= 1, out non-null");
  int dev = 0, smem_optin = 0, sms = 0;
  TV_CUDA(cudaGetDevice(&dev));
  TV_CUDA(cudaDeviceGetAttribute(&smem_optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev));
  TV_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
  const int N = n_states;
  // the grid plan's own matvec layout for this shape (row padding, split)
  tv::GridParams P;
  std::vector<long long> wr;
  std::vector<int> first, count, base;
  int Np = (N + 15) / 16 * 16, split = 0;
  if (plan_grid_nd(N, std::max(max_dur, 9), sms, smem_optin, false, P, wr, first, count, base)) {
    Np = P.Np;
    split = P.cs_split;
  }
  const int cs = (N + 31) / 32 * 32;
  const int threads = cs * (split ? 2 : 1);
  const size_t bytes = (size_t)4 * N * (Np + 4) + 8 * Np + 32 * N + 8 * (size_t)N * N + 12 * Np;
  if (bytes > (size_t)smem_optin) return fail(TV_ETOOBIG, "tv_step_floor: tables exceed shared memory");
  int rc;
  if ((rc = raise_smem_limit((const void*)tv::floor_chain_kernel)) != TV_OK) return rc;
  // transition scores of the benchmark family's range (log of Dirichlet rows)
  std::vector<double> tr((size_t)N * N);
  uint64_t x = 0x9e3779b97f4a7c15ull;
  for (auto& v : tr) {
    x ^= x << 13; x ^= x >> 7; x ^= x << 17;
    v = std::log(1e-6 + (double)(x >> 11) * 0x1.0p-53);
  }
  struct Bufs {
    double* tr = nullptr;
    long long* out = nullptr;
    unsigned long long* words = nullptr;
    int* status = nullptr;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    ~Bufs() {
      cudaFree(tr); cudaFree(out); cudaFree(words); cudaFree(status);
      if (e0) cudaEventDestroy(e0);
      if (e1) cudaEventDestroy(e1);
    }
  } b;
  TV_CUDA(cudaMalloc(&b.tr, sizeof(double) * tr.size()));
  TV_CUDA(cudaMalloc(&b.out, sizeof(long long) * 8));
  TV_CUDA(cudaMalloc(&b.words, sizeof(unsigned long long) * 4));
  TV_CUDA(cudaMalloc(&b.status, sizeof(int)));
  TV_CUDA(cudaMemcpy(b.tr, tr.data(), sizeof(double) * tr.size(), cudaMemcpyHostToDevice));
  TV_CUDA(cudaMemset(b.out, 0, sizeof(long long) * 8));
  TV_CUDA(cudaMemset(b.words, 0, sizeof(unsigned long long) * 4));
  TV_CUDA(cudaMemset(b.status, 0, sizeof(int)));
  TV_CUDA(cudaEventCreate(&b.e0));
  TV_CUDA(cudaEventCreate(&b.e1));
  const int f = 20;
  const double scale = std::ldexp(1.0, f);
  // warm-up, then the timed chain
  tv::floor_chain_kernel<<<1, threads, bytes>>>(N, Np, split, std::min<int64_t>(steps, 1000), b.tr, scale,
                                                f - tv::COARSE_F, b.out);
  TV_CUDA(cudaGetLastError());
  TV_CUDA(cudaEventRecord(b.e0));
  tv::floor_chain_kernel<<<1, threads, bytes>>>(N, Np, split, steps, b.tr, scale, f - tv::COARSE_F, b.out);
  TV_CUDA(cudaGetLastError());
  TV_CUDA(cudaEventRecord(b.e1));
  TV_CUDA(cudaEventSynchronize(b.e1));
  long long hout[8] = {0};
  TV_CUDA(cudaMemcpy(hout, b.out, sizeof(hout), cudaMemcpyDeviceToHost));
  float ms = 0.0f;
  TV_CUDA(cudaEventElapsedTime(&ms, b.e0, b.e1));
  out[0] = (double)hout[0] / (double)steps;
  out[1] = 1e3 * (double)ms / (double)steps;
  // cross-SM round trip: one CTA per SM, CTA 0 and the last one
  const size_t rt_smem = (size_t)smem_optin / 2 + 1024;
  if ((rc = raise_smem_limit((const void*)tv::xsm_roundtrip_kernel)) != TV_OK) return rc;
  const int iters = 2000;
  long long limit = 1LL << 31;
  void* args[] = {&b.words, (void*)&iters, &limit, &b.out, &b.status};
  TV_CUDA(cudaMemset(b.out, 0, sizeof(long long) * 8));
  TV_CUDA(cudaLaunchCooperativeKernel((const void*)tv::xsm_roundtrip_kernel, dim3(sms), dim3(32), args, rt_smem,
                                      nullptr));
  TV_CUDA(cudaDeviceSynchronize());
  int st = 0;
  TV_CUDA(cudaMemcpy(&st, b.status, sizeof(int), cudaMemcpyDeviceToHost));
  TV_CUDA(cudaMemcpy(hout, b.out, sizeof(hout), cudaMemcpyDeviceToHost));
  if (st != 0) return fail(TV_ETIMEOUT, "tv_step_floor: the cross-SM round trip timed out");
  out[2] = (double)hout[0] / iters;
  out[3] = out[2] * out[1] / std::max(out[0], 1e-9);
  out[4] = (double)split;
  out[5] = (double)hout[1];
  out[6] = (double)hout[2];
  return TV_OK;
}

}  // extern "C"

#include "tv_server.cuh"
