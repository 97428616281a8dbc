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
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include "../../include/tv_gb300.h"
#include "tv_cta.cuh"

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

template <class T>
struct DevBuf {
  T* p = nullptr;
  size_t n = 0;
  int ensure(size_t count) {
    if (count <= n && p) return TV_OK;
    if (p) cudaFree(p);
    p = nullptr;
    n = 0;
    if (count == 0) count = 1;
    cudaError_t e = cudaMalloc(&p, count * sizeof(T));
    if (e != cudaSuccess) {
      p = nullptr;
      return fail(TV_ENOMEM, std::string("cudaMalloc: ") + cudaGetErrorString(e));
    }
    n = count;
    return TV_OK;
  }
  void release() {
    if (p) cudaFree(p);
    p = nullptr;
    n = 0;
  }
};

constexpr int kThreads = 256;

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
  DevBuf<unsigned char> scratch;
  DevBuf<int32_t> obs_tmp, path_tmp;
  DevBuf<double> ll_tmp;
  int64_t last_launches = 0;
  int sm_count = 0;
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
  tv::ModelView v;
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
                 int32_t* path_dev, double* ll_dev, cudaStream_t st) {
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

  tv::CtaLayout L = tv::make_cta_layout(N, D);
  int dev = 0;
  TV_CUDA(cudaGetDevice(&dev));
  int smem_optin = 0;
  TV_CUDA(cudaDeviceGetAttribute(&smem_optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev));
  auto kern = tv::cta_decode_kernel<kThreads>;
  size_t dyn = 0;
  const size_t static_smem = 64;
  if (L.bytes + static_smem <= (size_t)smem_optin) {
    L.in_smem = 1;
    dyn = L.bytes;
    TV_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)dyn));
  }
  int per_sm = 1;
  TV_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, kThreads, dyn));
  per_sm = std::max(per_sm, 1);
  int grid = std::min(n_seq, m->sm_count * per_sm);
  grid = std::max(grid, 1);
  unsigned char* scratch = nullptr;
  if (!L.in_smem) {
    if ((rc = m->scratch.ensure((size_t)grid * L.bytes)) != TV_OK) return rc;
    scratch = m->scratch.p;
  }
  tv::BatchView bv;
  bv.obs = obs_dev;
  bv.off = m->off.p;
  bv.path = path_dev;
  bv.loglik = ll_dev;
  bv.psi = m->psi.p;
  bv.status = m->status.p;
  bv.next = m->counter.p;
  bv.n_seq = n_seq;
  kern<<<grid, kThreads, dyn, st>>>(view(m, Q), bv, L, scratch);
  TV_CUDA(cudaGetLastError());
  m->last_launches += 1;
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

}  // namespace

extern "C" {

const char* tv_last_error(void) { return g_err.c_str(); }

int tv_model_create(int N, int O, int D, const double* trans, const double* emission,
                    const double* dur_lin, const double* start, const double* dur, tv_model* out) {
  (void)dur_lin;
  if (!out) return fail(TV_EINVAL, "out is null");
  *out = nullptr;
  if (N <= 0 || O <= 0 || D <= 0) return fail(TV_EINVAL, "n_states, n_symbols and max_dur must be positive");
  if (N > 32768 || D > 65536) return fail(TV_ETOOBIG, "n_states must be <= 32768 and max_dur <= 65536");
  if (!trans || !emission || !start || !dur) return fail(TV_EINVAL, "null model table");
  tv_model_s* m = new tv_model_s();
  m->N = N; m->O = O; m->D = D;
  if (!all_finite(trans, (size_t)N * N, &m->tmax) || !all_finite(emission, (size_t)O * N, &m->emax) ||
      !all_finite(start, (size_t)N, &m->smax) || !all_finite(dur, (size_t)D * N, &m->dmax)) {
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
  if (e == cudaSuccess) e = cudaMemcpy(m->em.p, emission, sizeof(double) * O * N, cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemcpy(m->trans.p, trans, sizeof(double) * N * N, cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemcpy(m->start.p, start, sizeof(double) * N, cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemcpy(m->durT.p, durT.data(), sizeof(double) * N * D, cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemcpy(m->survT.p, survT.data(), sizeof(double) * N * D, cudaMemcpyHostToDevice);
  if (e != cudaSuccess) {
    tv_model_destroy(m);
    return fail(TV_ECUDA, std::string("model upload: ") + cudaGetErrorString(e));
  }
  *out = m;
  return TV_OK;
}

int tv_model_destroy(tv_model m) {
  if (!m) return TV_OK;
  m->em.release(); m->trans.release(); m->start.release(); m->durT.release(); m->survT.release();
  m->qem.release(); m->qtr.release(); m->qdurT.release();
  m->psi.release(); m->status.release(); m->counter.release(); m->off.release(); m->scratch.release();
  m->obs_tmp.release(); m->path_tmp.release(); m->ll_tmp.release();
  delete m;
  return TV_OK;
}

int64_t tv_model_last_launches(tv_model m) { return m ? m->last_launches : 0; }

int tv_decode_device(tv_model m, const int32_t* obs_dev, int64_t T, int32_t* path_dev, double* ll_dev,
                     void* stream) {
  if (!m || !obs_dev || !path_dev) return fail(TV_EINVAL, "null argument");
  if (T <= 0 || T > 0x7fffffffLL) return fail(TV_ETOOBIG, "T must be in [1, 2^31-1]");
  std::lock_guard<std::mutex> lk(m->mu);
  m->last_launches = 0;
  const int64_t off[2] = {0, T};
  return launch_batch(m, 1, off, obs_dev, path_dev, ll_dev, (cudaStream_t)stream);
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
  const int64_t off[2] = {0, T};
  if ((rc = launch_batch(m, 1, off, m->obs_tmp.p, m->path_tmp.p, m->ll_tmp.p, st)) != TV_OK) return rc;
  TV_CUDA(cudaMemcpyAsync(path_out, m->path_tmp.p, sizeof(int32_t) * T, cudaMemcpyDeviceToHost, st));
  double ll = 0;
  TV_CUDA(cudaMemcpyAsync(&ll, m->ll_tmp.p, sizeof(double), cudaMemcpyDeviceToHost, st));
  if ((rc = read_status(m, 1, st)) != TV_OK) return rc;
  if (loglik_out) *loglik_out = ll;
  return TV_OK;
}

int tv_decode_batch_device(tv_model m, int n_seq, const int64_t* offsets, const int32_t* obs_dev,
                           int32_t* path_dev, double* ll_dev, void* stream) {
  if (!m || !offsets || !obs_dev || !path_dev || n_seq <= 0) return fail(TV_EINVAL, "bad argument");
  std::lock_guard<std::mutex> lk(m->mu);
  m->last_launches = 0;
  if (offsets[0] != 0) return fail(TV_EINVAL, "offsets[0] must be 0");
  return launch_batch(m, n_seq, offsets, obs_dev, path_dev, ll_dev, (cudaStream_t)stream);
}

int tv_decode_batch(tv_model m, int n_seq, const int64_t* offsets, const int32_t* obs, int32_t* path,
                    double* loglik_out) {
  if (!m || !offsets || !obs || !path || n_seq <= 0) return fail(TV_EINVAL, "bad argument");
  if (offsets[0] != 0) return fail(TV_EINVAL, "offsets[0] must be 0");
  for (int k = 0; k < n_seq; ++k)
    if (offsets[k + 1] <= offsets[k]) return fail(TV_EINVAL, "offsets must increase");
  const int64_t total = offsets[n_seq];
  int rc = check_obs_host(obs, total, m->O);
  if (rc != TV_OK) return rc;
  std::lock_guard<std::mutex> lk(m->mu);
  m->last_launches = 0;
  cudaStream_t st = 0;
  if ((rc = m->obs_tmp.ensure((size_t)total)) != TV_OK) return rc;
  if ((rc = m->path_tmp.ensure((size_t)total)) != TV_OK) return rc;
  if ((rc = m->ll_tmp.ensure((size_t)n_seq)) != TV_OK) return rc;
  TV_CUDA(cudaMemcpyAsync(m->obs_tmp.p, obs, sizeof(int32_t) * total, cudaMemcpyHostToDevice, st));
  if ((rc = launch_batch(m, n_seq, offsets, m->obs_tmp.p, m->path_tmp.p, m->ll_tmp.p, st)) != TV_OK) return rc;
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

}  // extern "C"
