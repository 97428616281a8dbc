// tv_server.cuh -- the decode server: continuous batching of independent
// requests, each with its own model (no reference counterpart; the reference
// decodes one sequence per blocking call, src/hsmm.cu:604-720).
//
// A scheduler thread owns all device work.  Submissions are copied and
// queued; the scheduler admits them in arrival order while the device-memory
// budget allows (model tables, back-pointers T*N, the D-deep window and the
// kernel's scratch, estimated from the shapes) and a stream is free.  Each
// admitted request gets its own model, buffers and stream, all allocated in
// that stream's order from the device memory pool, so requests overlap on the
// GPU and finishing one never synchronises the device.  Windows that fit one
// CTA's shared memory run on the one-CTA kernel; larger ones on the grid
// kernel with only as many CTAs as the window needs (so several run side by
// side).  Completions are found by event queries; results are copied out and
// the request's memory returns to the budget.  Each request runs the same
// kernels on the same inputs as a decode alone, so its result does not depend
// on what else is in flight.
//
// This file is included by tv_host.cu (it uses that file's internals).
#pragma once
#include <atomic>
#include <chrono>
#include <condition_variable>
#include <deque>
#include <thread>
#include <unordered_map>

struct tv_server_s;

namespace {

struct SrvRequest {
  int64_t ticket = 0;
  int N = 0, O = 0, D = 0;
  int64_t T = 0;
  bool gaussian = false;
  std::vector<double> trans, em, start, dur, x, mean, sd;
  std::vector<int32_t> obs;
  // results
  std::vector<int32_t> path;
  double ll = 0.0;
  int status = TV_OK;
  std::string error;
  double t_submit = 0, t_admit = 0, t_done = 0;  // ms since the server started
  size_t bytes = 0;
  int grid_ctas = 0;  // > 0: decoded on a grid of this many CTAs (chosen at admission for latency)
  int sms = 0;        // SMs the request is counted as holding while it runs
  // in flight
  tv_model m = nullptr;
  cudaStream_t st = nullptr;
  cudaEvent_t ev = nullptr;
  int32_t* obs_dev = nullptr;
  int32_t* path_dev = nullptr;
  double* ll_dev = nullptr;
};

// Device bytes a request holds while in flight (an upper estimate).
size_t request_bytes(const SrvRequest& r, bool grid, int G) {
  const size_t N = r.N, O = r.O, D = r.D, T = r.T;
  size_t b = 16 * O * N + 16 * N * N + 8 * N + 24 * N * D  // exact + fixed-point tables, survival
             + 4 * T * N + 8 * T + 64 * 1024;               // back-pointers, obs + path, small scratch
  if (r.gaussian) b += 8 * T + 8 * T * N;                   // observations and the front-end's table
  if (grid) {
    b += 8 * T * tv::GRID_L * N;                           // window sums of the head's candidates
    b += 8 * D * ((D + tv::CK_STRIDE - 1) / tv::CK_STRIDE + 1) * N;  // checkpoints of the early window sums
    b += 8 * D * N;                                          // initialisation scores
    b += 48 * D * N + 256 * (size_t)G;                       // worker windows when they are kept in L2
    b += 8 * ((size_t)tv::SLOT_RING * N * tv::SLOT_WORDS + (size_t)tv::PART_RING * (G + N) * tv::MSG_WORDS +
              (D + 2 * tv::GRID_L + 8) * N * 2);
  }
  return b;
}

double now_ms(std::chrono::steady_clock::time_point t0) {
  return std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
}

// Smallest grid (head + workers) whose workers hold the window in shared
// memory, times `spread` for speed; 0 if none.
int grid_ctas_nd(int N, int D, int sm_count, int smem_optin, double spread) {
  std::vector<int> first, count, base;
  std::vector<long long> wr;
  tv::GridParams P;
  for (int G = 2; G <= sm_count; ++G) {
    if (plan_grid_nd(N, D, G, smem_optin, false, P, wr, first, count, base) && !P.w_global)
      return std::min(sm_count, std::max(G, (int)std::ceil(G * spread)));
  }
  return 0;
}

int grid_ctas_for(tv_model_s* m, int smem_optin, double spread) {
  return grid_ctas_nd(m->N, m->D, m->sm_count, smem_optin, spread);
}

// Latency mode: while the device has SMs to spare and nothing else waits, a
// long request is decoded on a grid of about 600 window cells per worker
// (measured on GB300: at N=50, D=100 a step takes 13.2 us on one CTA, 2.8 us
// on 16 CTAs; at N=50, D=1000, 2.8 us on the 24 CTAs its window needs and
// 1.4 us on 96), at least the smallest grid that holds its window, at most
// 96 CTAs.  This spends more SM time per request than the one-CTA kernel or
// the smallest grid, so it is only taken below the load threshold; under load
// the throughput-first choice stands.
constexpr double kLatencyMinCells = 2e8;  // T*N*D below this finishes in tens of ms anyway
int latency_grid_ctas(int N, int D, int sm_count, int smem_optin) {
  const int g_min = grid_ctas_nd(N, D, sm_count, smem_optin, 1.0);
  if (g_min <= 0) return 0;
  const long long want = (long long)N * D / 600 + 2;
  return (int)std::min<long long>(std::min(96, sm_count), std::max<long long>(g_min, want));
}

}  // namespace

struct tv_server_s {
  std::mutex mu;
  std::condition_variable cv;
  std::deque<SrvRequest*> pending;
  std::vector<SrvRequest*> running;
  std::unordered_map<int64_t, SrvRequest*> finished;
  std::unordered_map<int64_t, int> state;  // 0 pending/running, 1 finished
  int64_t next_ticket = 0;
  size_t budget = 0, in_use = 0, peak = 0;
  int64_t admitted = 0, completed = 0, failed = 0;
  std::vector<cudaStream_t> streams;
  std::vector<cudaEvent_t> events;
  std::vector<int> free_slots;
  std::thread th;
  bool stop = false;
  bool hold = false;  // admission paused until the next completion
  uint64_t pool_keep_before = 0;  // the pool's retention setting before this server
  int dev = 0, smem_optin = 0, sm_count = 0;
  int sms_busy = 0;  // SMs counted as held by the admitted requests
  std::chrono::steady_clock::time_point t0 = std::chrono::steady_clock::now();

  // ---- scheduler thread ----
  void start_request(SrvRequest* r) {
    g_alloc_async = true;
    g_alloc_stream = r->st;
    int rc = TV_OK;
    if (r->gaussian)
      rc = model_create_gaussian(r->N, r->D, r->T, r->trans.data(), r->start.data(), r->dur.data(), r->x.data(),
                                 r->mean.data(), r->sd.data(), &r->m);
    else
      rc = model_create_impl(r->N, r->O, r->D, r->trans.data(), r->em.data(), nullptr, r->start.data(),
                             r->dur.data(), &r->m);
    if (rc == TV_OK) {
      const tv::CtaLayout L = tv::make_cta_layout(r->N, r->D);
      if (r->grid_ctas > 0) {
        r->m->path_pref = TV_PATH_GRID;  // latency mode (admission chose the grid)
        r->m->grid_ctas = r->grid_ctas;
      } else if (L.bytes + 64 > (size_t)smem_optin) {
        const int G = grid_ctas_for(r->m, smem_optin, 1.5);
        r->m->path_pref = TV_PATH_GRID;
        r->m->grid_ctas = G;  // 0 (none fits shared memory): the whole GPU with the window in L2
      }
    }
    cudaError_t e = cudaSuccess;
    if (rc == TV_OK) {
      e = cudaMallocAsync((void**)&r->obs_dev, sizeof(int32_t) * r->T, r->st);
      if (e == cudaSuccess) e = cudaMallocAsync((void**)&r->path_dev, sizeof(int32_t) * r->T, r->st);
      if (e == cudaSuccess) e = cudaMallocAsync((void**)&r->ll_dev, sizeof(double), r->st);
      if (e == cudaSuccess) {
        if (r->gaussian) {
          iota_kernel<<<(unsigned)std::min<int64_t>((r->T + 255) / 256, 4096), 256, 0, r->st>>>(r->obs_dev, r->T);
          e = cudaGetLastError();
        } else {
          e = cudaMemcpyAsync(r->obs_dev, r->obs.data(), sizeof(int32_t) * r->T, cudaMemcpyHostToDevice, r->st);
        }
      }
      if (e != cudaSuccess) {
        cudaGetLastError();
        rc = fail(TV_ENOMEM, std::string("request buffers: ") + cudaGetErrorString(e));
      }
    }
    if (rc == TV_OK) {
      std::lock_guard<std::mutex> lk(r->m->mu);
      r->m->last_launches = 0;
      rc = launch_single(r->m, r->obs_dev, r->T, r->path_dev, r->ll_dev, r->st);
    }
    if (rc != TV_OK) {
      r->status = rc;
      r->error = g_err;
    }
    cudaEventRecord(r->ev, r->st);
    g_alloc_async = false;
  }

  // Frees a request's device memory (in its stream's order).
  void release_request(SrvRequest* r) {
    g_alloc_async = true;
    g_alloc_stream = r->st;
    if (r->obs_dev) cudaFreeAsync(r->obs_dev, r->st);
    if (r->path_dev) cudaFreeAsync(r->path_dev, r->st);
    if (r->ll_dev) cudaFreeAsync(r->ll_dev, r->st);
    r->obs_dev = r->path_dev = nullptr;
    r->ll_dev = nullptr;
    if (r->m) tv_model_destroy(r->m);
    r->m = nullptr;
    g_alloc_async = false;
  }

  void finish_request(SrvRequest* r) {
    g_alloc_async = true;
    g_alloc_stream = r->st;
    if (r->status == TV_OK) {
      int rc = (r->m->last_path == TV_PATH_GRID) ? read_grid_status(r->m, r->st) : read_status(r->m, 1, r->st);
      if (rc == TV_OK) {
        r->path.resize((size_t)r->T);
        cudaError_t e = cudaMemcpyAsync(r->path.data(), r->path_dev, sizeof(int32_t) * r->T, cudaMemcpyDeviceToHost, r->st);
        if (e == cudaSuccess) e = cudaMemcpyAsync(&r->ll, r->ll_dev, sizeof(double), cudaMemcpyDeviceToHost, r->st);
        if (e == cudaSuccess) e = cudaStreamSynchronize(r->st);
        if (e != cudaSuccess) rc = fail(TV_ECUDA, std::string("result copy: ") + cudaGetErrorString(e));
      }
      if (rc != TV_OK) {
        r->status = rc;
        r->error = g_err;
      }
    }
    g_alloc_async = false;
    release_request(r);
    // free the inputs; keep the results
    std::vector<double>().swap(r->trans); std::vector<double>().swap(r->em); std::vector<double>().swap(r->x);
    std::vector<int32_t>().swap(r->obs);
  }

  void loop() {
    cudaSetDevice(dev);
    for (;;) {
      bool progress = false;
      std::vector<SrvRequest*> to_start;
      {
        std::unique_lock<std::mutex> lk(mu);
        if (stop && pending.empty() && running.empty()) return;
        if (pending.empty() && running.empty()) {
          cv.wait_for(lk, std::chrono::milliseconds(50));
          continue;
        }
        // admission in arrival order while memory and a stream allow (a
        // request alone on an idle device is always admitted); after a
        // placement failure, wait for a completion first
        while (!hold && !pending.empty() && !free_slots.empty()) {
          SrvRequest* r = pending.front();
          const bool big = tv::make_cta_layout(r->N, r->D).bytes + 64 > (size_t)smem_optin;
          // latency mode when this request is the only one waiting and the
          // SMs it would take are free (three quarters of the device at most)
          int gl = 0;
          if (pending.size() == 1 && (double)r->T * r->N * r->D >= kLatencyMinCells) {
            gl = latency_grid_ctas(r->N, r->D, sm_count, smem_optin);
            if (gl > 0 && sms_busy + gl > (3 * sm_count) / 4) gl = 0;
          }
          const int g_def = big ? std::max(1, grid_ctas_nd(r->N, r->D, sm_count, smem_optin, 1.5)) : 1;
          const size_t need = request_bytes(*r, big || gl > 0, gl > 0 ? gl : (big ? g_def : 16));
          if (in_use + need > budget && !(running.empty() && to_start.empty())) break;
          pending.pop_front();
          r->grid_ctas = gl;
          r->sms = gl > 0 ? gl : g_def;
          sms_busy += r->sms;
          const int slot = free_slots.back();
          free_slots.pop_back();
          r->st = streams[slot];
          r->ev = events[slot];
          r->bytes = need;
          r->t_admit = now_ms(t0);
          in_use += need;
          peak = std::max(peak, in_use);
          ++admitted;
          to_start.push_back(r);
        }
      }
      for (size_t q = 0; q < to_start.size(); ++q) {
        SrvRequest* r = to_start[q];
        start_request(r);
        std::lock_guard<std::mutex> lk(mu);
        if (r->status == TV_ENOMEM && !running.empty()) {
          // The estimate let it in but the device could not place it (the
          // pool's free blocks are fragmented): give the memory back, trim
          // the pool and retry it first once another request completes.
          cudaStreamSynchronize(r->st);
          release_request(r);
          cudaStreamSynchronize(r->st);
          cudaMemPool_t pool;
          if (cudaDeviceGetDefaultMemPool(&pool, dev) == cudaSuccess) cudaMemPoolTrimTo(pool, 0);
          r->status = TV_OK;
          r->error.clear();
          in_use -= r->bytes;
          sms_busy -= r->sms;
          r->sms = 0;
          for (size_t s2 = 0; s2 < streams.size(); ++s2)
            if (streams[s2] == r->st) free_slots.push_back((int)s2);
          r->st = nullptr;
          r->ev = nullptr;
          --admitted;
          // this one and the rest of this admission pass go back in arrival order
          for (size_t q2 = to_start.size(); q2-- > q + 1;) {
            SrvRequest* o = to_start[q2];
            in_use -= o->bytes;
            sms_busy -= o->sms;
            o->sms = 0;
            for (size_t s2 = 0; s2 < streams.size(); ++s2)
              if (streams[s2] == o->st) free_slots.push_back((int)s2);
            o->st = nullptr;
            o->ev = nullptr;
            --admitted;
            pending.push_front(o);
          }
          pending.push_front(r);
          hold = true;
          progress = true;
          break;
        }
        running.push_back(r);
        progress = true;
      }
      // completions
      std::vector<SrvRequest*> done_now;
      {
        std::lock_guard<std::mutex> lk(mu);
        for (size_t k = 0; k < running.size();) {
          if (cudaEventQuery(running[k]->ev) == cudaSuccess) {
            done_now.push_back(running[k]);
            running[k] = running.back();
            running.pop_back();
          } else {
            ++k;
          }
        }
      }
      for (SrvRequest* r : done_now) {
        finish_request(r);
        r->t_done = now_ms(t0);
        std::lock_guard<std::mutex> lk(mu);
        in_use -= r->bytes;
        sms_busy -= r->sms;
        for (size_t s = 0; s < streams.size(); ++s)
          if (streams[s] == r->st) free_slots.push_back((int)s);
        r->st = nullptr;
        r->ev = nullptr;
        finished[r->ticket] = r;
        state[r->ticket] = 1;
        if (r->status == TV_OK) ++completed;
        else ++failed;
        progress = true;
      }
      if (!done_now.empty()) {
        hold = false;
        cv.notify_all();
      }
      if (!progress) std::this_thread::sleep_for(std::chrono::microseconds(50));
    }
  }
};

extern "C" {

tv_server tv_server_create(int64_t budget_bytes, int max_inflight) {
  int devs = 0;
  if (cudaGetDeviceCount(&devs) != cudaSuccess || devs == 0) {
    fail(TV_ENODEV, "no CUDA device");
    return nullptr;
  }
  if (max_inflight <= 0) max_inflight = 64;
  tv_server_s* s = new tv_server_s();
  cudaGetDevice(&s->dev);
  cudaDeviceGetAttribute(&s->smem_optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, s->dev);
  cudaDeviceGetAttribute(&s->sm_count, cudaDevAttrMultiProcessorCount, s->dev);
  size_t free_b = 0, total_b = 0;
  cudaMemGetInfo(&free_b, &total_b);
  s->budget = budget_bytes > 0 ? (size_t)budget_bytes : (size_t)(0.8 * (double)free_b);
  // Keep part of the freed pool memory for reuse instead of returning it at
  // each synchronisation (a property of this process's pool); the rest goes
  // back, which bounds fragmentation.
  cudaMemPool_t pool;
  if (cudaDeviceGetDefaultMemPool(&pool, s->dev) == cudaSuccess) {
    cudaMemPoolGetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &s->pool_keep_before);
    uint64_t keep = s->budget / 4;
    cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &keep);
  }
  for (int k = 0; k < max_inflight; ++k) {
    cudaStream_t st;
    cudaEvent_t ev;
    if (cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking) != cudaSuccess ||
        cudaEventCreateWithFlags(&ev, cudaEventDisableTiming) != cudaSuccess) {
      fail(TV_ECUDA, "stream or event creation failed");
      break;
    }
    s->streams.push_back(st);
    s->events.push_back(ev);
    s->free_slots.push_back(k);
  }
  if (s->streams.empty()) {
    delete s;
    return nullptr;
  }
  // the one-CTA kernel's shared-memory limit, raised before any concurrent launch
  raise_smem_limit((const void*)tv::cta_decode_kernel<kThreads>);
  s->th = std::thread([s] { s->loop(); });
  return s;
}

int tv_server_destroy(tv_server s) {
  if (!s) return TV_OK;
  {
    std::lock_guard<std::mutex> lk(s->mu);
    s->stop = true;
  }
  s->cv.notify_all();
  if (s->th.joinable()) s->th.join();
  for (auto& kv : s->finished) delete kv.second;
  for (cudaStream_t st : s->streams) {
    cudaStreamSynchronize(st);
    cudaStreamDestroy(st);
  }
  for (cudaEvent_t ev : s->events) cudaEventDestroy(ev);
  // hand the pool's memory back and restore its retention setting
  cudaMemPool_t pool;
  if (cudaDeviceGetDefaultMemPool(&pool, s->dev) == cudaSuccess) {
    cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &s->pool_keep_before);
    cudaMemPoolTrimTo(pool, 0);
  }
  delete s;
  return TV_OK;
}

static int64_t srv_enqueue(tv_server s, SrvRequest* r) {
  std::lock_guard<std::mutex> lk(s->mu);
  if (s->stop) {
    delete r;
    return fail(TV_EINVAL, "server is stopping");
  }
  r->ticket = s->next_ticket++;
  r->t_submit = now_ms(s->t0);
  s->state[r->ticket] = 0;
  s->pending.push_back(r);
  s->cv.notify_all();
  return r->ticket;
}

int64_t tv_server_submit(tv_server s, int n_states, int n_symbols, int max_dur, int64_t T, const double* trans,
                         const double* emission, const double* dur_lin, const double* start, const double* dur,
                         const int32_t* obs) {
  (void)dur_lin;
  if (!s || !trans || !emission || !start || !dur || !obs) return fail(TV_EINVAL, "null argument");
  if (n_states <= 0 || n_symbols <= 0 || max_dur <= 0) return fail(TV_EINVAL, "sizes must be positive");
  if (T <= 0 || T > 0x7fffffffLL) return fail(TV_ETOOBIG, "T must be in [1, 2^31-1]");
  if (T < max_dur)
    return fail(TV_ESHORT, "T=" + std::to_string(T) + " < D=" + std::to_string(max_dur) +
                               "; the reference initialisation needs T >= D");
  int rc = check_obs_host(obs, T, n_symbols);
  if (rc != TV_OK) return rc;
  SrvRequest* r = new SrvRequest();
  r->N = n_states; r->O = n_symbols; r->D = max_dur; r->T = T;
  r->trans.assign(trans, trans + (size_t)n_states * n_states);
  r->em.assign(emission, emission + (size_t)n_symbols * n_states);
  r->start.assign(start, start + n_states);
  r->dur.assign(dur, dur + (size_t)max_dur * n_states);
  r->obs.assign(obs, obs + T);
  return srv_enqueue(s, r);
}

int64_t tv_server_submit_gaussian(tv_server s, int n_states, int max_dur, int64_t T, const double* trans,
                                  const double* dur_lin, const double* start, const double* dur, const double* x,
                                  const double* mean, const double* sd) {
  (void)dur_lin;
  if (!s || !trans || !start || !dur || !x || !mean || !sd) return fail(TV_EINVAL, "null argument");
  if (n_states <= 0 || max_dur <= 0) return fail(TV_EINVAL, "sizes must be positive");
  if (T <= 0 || T > 0x7fffffffLL) return fail(TV_ETOOBIG, "T must be in [1, 2^31-1]");
  if (T < max_dur)
    return fail(TV_ESHORT, "T=" + std::to_string(T) + " < D=" + std::to_string(max_dur) +
                               "; the reference initialisation needs T >= D");
  SrvRequest* r = new SrvRequest();
  r->gaussian = true;
  r->N = n_states; r->O = (int)T; r->D = max_dur; r->T = T;
  r->trans.assign(trans, trans + (size_t)n_states * n_states);
  r->start.assign(start, start + n_states);
  r->dur.assign(dur, dur + (size_t)max_dur * n_states);
  r->x.assign(x, x + T);
  r->mean.assign(mean, mean + n_states);
  r->sd.assign(sd, sd + n_states);
  return srv_enqueue(s, r);
}

static int srv_take(tv_server s, int64_t ticket, int32_t* path_out, double* loglik_out, double* latency_ms_out,
                    bool block) {
  std::unique_lock<std::mutex> lk(s->mu);
  auto it = s->state.find(ticket);
  if (it == s->state.end()) return fail(TV_EINVAL, "unknown ticket " + std::to_string(ticket));
  if (it->second == 0) {
    if (!block) return 0;
    s->cv.wait(lk, [&] { return s->state[ticket] == 1; });
  }
  SrvRequest* r = s->finished[ticket];
  s->finished.erase(ticket);
  s->state.erase(ticket);
  lk.unlock();
  int rc = r->status;
  if (rc == TV_OK) {
    if (path_out) std::memcpy(path_out, r->path.data(), sizeof(int32_t) * r->T);
    if (loglik_out) *loglik_out = r->ll;
    if (latency_ms_out) {
      latency_ms_out[0] = r->t_done - r->t_submit;
      latency_ms_out[1] = r->t_admit - r->t_submit;
    }
    rc = 1;
  } else {
    fail(r->status, r->error);
  }
  delete r;
  return rc;
}

int tv_server_poll(tv_server s, int64_t ticket, int32_t* path_out, double* loglik_out, double* latency_ms_out) {
  if (!s) return fail(TV_EINVAL, "null server");
  return srv_take(s, ticket, path_out, loglik_out, latency_ms_out, false);
}

int tv_server_wait(tv_server s, int64_t ticket, int32_t* path_out, double* loglik_out, double* latency_ms_out) {
  if (!s) return fail(TV_EINVAL, "null server");
  return srv_take(s, ticket, path_out, loglik_out, latency_ms_out, true);
}

int tv_server_stats(tv_server s, int64_t* out) {
  if (!s || !out) return fail(TV_EINVAL, "null argument");
  std::lock_guard<std::mutex> lk(s->mu);
  out[0] = s->admitted;
  out[1] = s->completed;
  out[2] = s->failed;
  out[3] = (int64_t)s->running.size();
  out[4] = (int64_t)s->pending.size();
  out[5] = (int64_t)s->in_use;
  out[6] = (int64_t)s->peak;
  out[7] = (int64_t)s->budget;
  return TV_OK;
}

int tv_gaussian_loglik(const double* x_dev, int64_t T, int n_states, const double* mean, const double* sd,
                       double* table_dev, void* stream) {
  return gaussian_table(x_dev, T, n_states, mean, sd, table_dev, (cudaStream_t)stream);
}

int tv_model_create_gaussian(int n_states, int max_dur, int64_t T, const double* trans, const double* dur_lin,
                             const double* start, const double* dur, const double* x, const double* mean,
                             const double* sd, tv_model* out) {
  (void)dur_lin;
  return model_create_gaussian(n_states, max_dur, T, trans, start, dur, x, mean, sd, out);
}

}  // extern "C"
